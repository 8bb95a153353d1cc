"""GPU tests of spg_multiply_to_host: the product computed in row blocks whose
device->host copies overlap later blocks must equal spg_multiply bit for bit
(and so the serial reference product, spgemm_common.cpp:131-178)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import csr_bits_equal, explain_diff, random_csr
from spgemm_gb300 import Csr, SpgError, synth_powerlaw, synth_uniform

pytestmark = pytest.mark.gpu


def to_host(engine, a, b, cap=None, pinned=False):
    import torch
    p = engine.scalar_multiplication_count(a, b) if cap is None else cap
    if pinned:
        rp = torch.empty(a.rows + 1, dtype=torch.int64, pin_memory=True)
        ci = torch.empty(max(p, 1), dtype=torch.int32, pin_memory=True)
        va = torch.empty(max(p, 1), dtype=torch.float64, pin_memory=True)
    else:
        rp, ci, va = np.empty(a.rows + 1, np.int64), np.empty(max(p, 1), np.int32), np.empty(max(p, 1), np.float64)
    nnz = engine.multiply_to_host(a, b, rp, ci, va)
    rp, ci, va = (np.asarray(x) for x in (rp, ci, va))
    return Csr(a.rows, b.cols, rp.copy(), ci[:nnz].copy(), va[:nnz].copy())


def test_small_product_matches_reference(engine, port):
    a = random_csr(300, 200, 12, 1)
    b = random_csr(200, 250, 9, 2)
    got = to_host(engine, a, b)
    want = port.serial_spgemm(a, b)
    assert csr_bits_equal(got, want), explain_diff(got, want)


@pytest.mark.parametrize("pinned", [False, True])
def test_row_blocks_match_single_call(engine, pinned):
    # 6.3 M entries in A: ten row blocks
    a = synth_powerlaw(262144, 24.0, 1.2, 20000, 2048, 0.7, seed=3)
    got = to_host(engine, a, a, pinned=pinned)
    assert engine.last_timings()["products"] == engine.scalar_multiplication_count(a, a)
    want = engine.multiply(a.to_device(), a.to_device(), out="device").download()
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_device_operands(engine):
    a = synth_uniform(30000, 30000, 4, 64, seed=5)
    b = synth_uniform(30000, 30000, 4, 64, seed=6)
    got = to_host(engine, a.to_device(), b.to_device(), cap=engine.scalar_multiplication_count(a, b))
    want = engine.multiply(a, b)
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_capacity_too_small(engine):
    a = random_csr(100, 80, 10, 3)
    b = random_csr(80, 90, 10, 4)
    nnz = engine.multiply(a, b).nnz
    with pytest.raises(SpgError) as e:
        to_host(engine, a, b, cap=nnz - 1)
    assert e.value.name == "SPG_BUDGET_EXCEEDED"
    got = to_host(engine, a, b, cap=nnz)  # exactly enough; the handle stays usable
    assert got.nnz == nnz


def test_empty_and_errors(engine):
    a = Csr.from_arrays(3, 4, [0, 0, 0, 0], [], [])
    b = random_csr(4, 5, 2, 1)
    got = to_host(engine, a, b, cap=0)
    assert got.nnz == 0 and got.row_ptr.tolist() == [0, 0, 0, 0]
    bad = Csr.from_arrays(2, 3, [0, 1, 2], [0, 7], [1.0, 1.0])
    with pytest.raises(SpgError) as e:
        to_host(engine, bad, Csr.from_arrays(3, 2, [0, 1, 2, 3], [0, 1, 0], [1.0, 1.0, 1.0]), cap=10)
    assert e.value.name == "SPG_OUT_OF_RANGE_COLUMN"


@pytest.mark.parametrize("pinned", [False, True])
def test_error_in_a_late_block_waits_for_earlier_copies(engine, pinned):
    # 6.3 M entries in A, so the product runs in ten row blocks; one A column in
    # the last rows points past B's rows, so the call fails in the last block,
    # after the copies of the earlier blocks into the host arrays have started.
    # The call must return only once those copies are done: the arrays do not
    # change after it returns, and the handle stays usable.
    import time
    import torch
    a = synth_powerlaw(262144, 24.0, 1.2, 20000, 2048, 0.7, seed=3)
    bad = Csr(a.rows, a.cols, a.row_ptr.copy(), a.col.copy(), a.val.copy())
    bad.col[int(bad.row_ptr[-2])] = a.cols  # last row: column == B.rows
    cap = engine.scalar_multiplication_count(a, a)
    if pinned:
        bufs = [torch.full((n,), -7, dtype=t, pin_memory=True)
                for n, t in ((a.rows + 1, torch.int64), (cap, torch.int32), (cap, torch.float64))]
    else:
        bufs = [np.full(a.rows + 1, -7, np.int64), np.full(cap, -7, np.int32), np.full(cap, -7.0, np.float64)]
    with pytest.raises(SpgError) as e:
        engine.multiply_to_host(bad, a, *bufs)
    assert e.value.name == "SPG_OUT_OF_RANGE_COLUMN"
    snap = [np.asarray(x).copy() for x in bufs]
    assert (snap[1] != -7).any(), "earlier blocks were copied out before the failing one"
    time.sleep(0.2)
    assert all(np.array_equal(np.asarray(x), s) for x, s in zip(bufs, snap))
    got = to_host(engine, a, a, pinned=pinned)
    want = engine.multiply(a.to_device(), a.to_device(), out="device").download()
    assert csr_bits_equal(got, want), explain_diff(got, want)
