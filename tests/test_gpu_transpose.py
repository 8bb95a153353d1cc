"""GPU transpose (spg_transpose): every row of A^T holds A's column in A's
row-major order (a stable sort by column), duplicates and explicit zeros
kept, values bit-identical."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import csr_bits_equal, explain_diff, random_csr
from spgemm_gb300 import Csr, synth_powerlaw, synth_restriction

pytestmark = pytest.mark.gpu


def stable_transpose(a: Csr) -> Csr:
    rows = np.repeat(np.arange(a.rows, dtype=np.int32), np.diff(a.row_ptr))
    order = np.argsort(a.col, kind="stable")
    rp = np.zeros(a.cols + 1, dtype=np.int64)
    np.cumsum(np.bincount(a.col, minlength=a.cols), out=rp[1:])
    return Csr(a.cols, a.rows, rp, rows[order].astype(np.int32), a.val[order])


@pytest.mark.parametrize("shape", [(1, 1), (7, 300), (300, 7), (500, 400), (2000, 3000)])
def test_random(engine, shape):
    m, n = shape
    rng = np.random.default_rng(m * 7 + n)
    a = random_csr(m, n, rng.integers(0, 25, size=m), m + n)  # unsorted rows, duplicates, explicit zeros
    got = engine.transpose(a)
    want = stable_transpose(a)
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_twice_restores_sorted_rows(engine):
    a = random_csr(800, 900, 12, 3, unsorted=False, duplicates=False)
    assert csr_bits_equal(engine.transpose(engine.transpose(a)), a)


def test_restriction_of_the_galerkin_chain(engine):
    r = synth_restriction(32)
    got = engine.transpose(r)
    want = synth_restriction(32, transpose=True)
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_full_size_powerlaw(engine):
    a = synth_powerlaw(1 << 20, 24.0, 1.2, 20000, 2048, 0.7, seed=1)
    r = engine.transpose(a.to_device(), out="device")
    got = r.download()
    r.free()
    want = stable_transpose(a)
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_empty_rows_and_matrix(engine):
    a = Csr.from_arrays(4, 6, [0, 0, 2, 2, 3], [5, 0, 5], [1.0, 2.0, 3.0])
    got = engine.transpose(a)
    assert got.row_ptr.tolist() == [0, 1, 1, 1, 1, 1, 3]
    assert got.col.tolist() == [1, 1, 3] and got.val.tolist() == [2.0, 1.0, 3.0]
    e = engine.transpose(Csr.from_arrays(3, 2, [0, 0, 0, 0], [], []))
    assert e.rows == 2 and e.cols == 3 and e.nnz == 0 and e.row_ptr.tolist() == [0, 0, 0]
