"""GPU tests of plans (spg_plan_*): the structure-dependent phases once, the
value-dependent ones replayed as a CUDA graph.  Every execution must equal
spg_multiply of the operands' current values bit for bit (the serial
reference product, spgemm_common.cpp:131-178), including after the values
change in place and when cancellation changes which entries survive."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import csr_bits_equal, explain_diff, random_csr, row_sizes_for_bins
from spgemm_gb300 import SpgError, synth_powerlaw

pytestmark = pytest.mark.gpu


def test_plan_matches_multiply_and_follows_new_values(engine, port):
    import torch
    a = random_csr(400, 300, 14, 1)
    b = random_csr(300, 350, 11, 2)
    da, db = a.to_device(), b.to_device()
    with engine.plan([(da, db)]) as plan:
        for step in range(3):
            nnz = plan.execute()
            got = plan.result(0)
            want = port.serial_spgemm(a, b)
            assert nnz == [want.nnz]
            assert csr_bits_equal(got, want), explain_diff(got, want)
            # new values in place (same structure): integers, so that some sums cancel
            rng = np.random.default_rng(step)
            a.val[:] = rng.integers(-2, 3, size=a.nnz).astype(np.float64)
            b.val[:] = rng.integers(-2, 3, size=b.nnz).astype(np.float64)
            da.val.copy_(torch.from_numpy(a.val))
            db.val.copy_(torch.from_numpy(b.val))
        assert plan.last_ms > 0


def test_plan_batch_of_uneven_products(engine):
    pairs = [row_sizes_for_bins(3), (random_csr(50, 40, 6, 4), random_csr(40, 60, 5, 5))]
    a = synth_powerlaw(20000, 24.0, 1.2, 3000, 256, 0.7, seed=9)
    pairs.append((a, a))
    dev = [(x.to_device(), y.to_device()) for x, y in pairs]
    with engine.plan(dev) as plan:
        nnz = plan.execute()
        for i, (x, y) in enumerate(pairs):
            want = engine.multiply(x, y)
            got = plan.result(i)
            assert nnz[i] == want.nnz
            assert csr_bits_equal(got, want), explain_diff(got, want)
        assert plan.execute() == nnz  # a replay reproduces it


def test_plan_errors(engine):
    a = random_csr(20, 10, 3, 1)
    b = random_csr(10, 12, 3, 2)
    with pytest.raises(TypeError):
        engine.plan([(a, b)])
    bad = random_csr(20, 10, 3, 1)
    bad.col[0] = 99
    with pytest.raises(SpgError) as e:
        engine.plan([(bad.to_device(), b.to_device())])
    assert e.value.name == "SPG_OUT_OF_RANGE_COLUMN"
    ok = engine.multiply(a, b)  # the handle stays usable
    assert ok.rows == 20
