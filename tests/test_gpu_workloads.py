"""Parity at the benchmark workloads' full sizes, through the C ABI.

* uniform 65,536^2 (16 distinct columns per row): every row bit for bit
  against the oracle's OpenMP restatement of the baseline spgemm().
* Galerkin chain on a 128^3 Laplacian: R*A and (R*A)*R^T bit for bit (dyadic
  values: every sum is exact).
* skewed power-law 1,048,576^2: every row's stored count against the
  reference's Partial criterion (row counts of the serial sums), sampled rows
  bit for bit (random rows plus the heaviest ones), the Full roundoff bound on
  sampled rows, and the exact power-of-two scaling property C(2A, A) = 2 C(A, A).
* rows at the limits of the packed (column, sequence) sort keys.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import csr_bits_equal, explain_diff
import spgemm_gb300 as sg

pytestmark = pytest.mark.gpu


def structure_ok(c) -> bool:
    lens = np.diff(c.row_ptr)
    if np.any(lens < 0) or c.row_ptr[0] != 0 or c.row_ptr[-1] != len(c.col):
        return False
    starts = np.zeros(len(c.col), dtype=bool)
    starts[c.row_ptr[:-1][lens > 0]] = True
    inc = np.diff(c.col.astype(np.int64)) > 0
    return bool(np.all(inc | starts[1:]) and np.all(c.val != 0) and np.all((c.col >= 0) & (c.col < c.cols)))


def rows_equal(c, want, rows) -> bool:
    for i, r in enumerate(rows):
        a0, a1 = c.row_ptr[r], c.row_ptr[r + 1]
        b0, b1 = want.row_ptr[i], want.row_ptr[i + 1]
        if a1 - a0 != b1 - b0 or not np.array_equal(c.col[a0:a1], want.col[b0:b1]):
            return False
        if not np.array_equal(c.val[a0:a1].view(np.uint64), want.val[b0:b1].view(np.uint64)):
            return False
    return True


@pytest.fixture(scope="module")
def powerlaw():
    return sg.synth_powerlaw(1 << 20, 24.0, 1.2, 20000, 2048, 0.7, seed=1)


@pytest.fixture(scope="module")
def powerlaw_product(engine, powerlaw):
    return engine.multiply(powerlaw, powerlaw)


def test_uniform_full(engine, port):
    a = sg.synth_uniform(65536, 65536, 16, seed=1)
    b = sg.synth_uniform(65536, 65536, 16, seed=2)
    got = engine.multiply(a, b)
    want = port.spgemm_omp(a, b)
    assert csr_bits_equal(got, want), explain_diff(got, want)
    assert engine.last_timings()["products"] == 16 * 16 * 65536


def test_galerkin_chain_full(engine, port):
    lap = sg.synth_laplacian3d(128)
    r = sg.synth_restriction(128)
    rt = sg.synth_restriction(128, transpose=True)
    ra = engine.multiply(r, lap)
    want_ra = port.spgemm_omp(r, lap)
    assert csr_bits_equal(ra, want_ra), explain_diff(ra, want_ra)
    assert ra.nnz == 8290304
    rar = engine.multiply(ra, rt)
    want = port.spgemm_omp(want_ra, rt)
    assert csr_bits_equal(rar, want), explain_diff(rar, want)
    assert rar.nnz == 1810432


def test_powerlaw_row_counts_partial(port, powerlaw, powerlaw_product):
    c = powerlaw_product
    assert structure_ok(c)
    ok, mismatches = port.compare_partial(*port.partial_reference(powerlaw, powerlaw), powerlaw.rows,
                                          powerlaw.cols, c)
    assert ok and mismatches == 0
    assert c.nnz == 583643070


def test_powerlaw_sampled_rows_bitwise(port, powerlaw, powerlaw_product):
    lens = np.diff(powerlaw.row_ptr)
    ub = np.zeros(powerlaw.rows, np.int64)
    np.add.at(ub, np.repeat(np.arange(powerlaw.rows), lens), lens[powerlaw.col])
    rng = np.random.default_rng(7)
    rows = np.unique(np.concatenate([rng.choice(powerlaw.rows, 400, replace=False), np.argsort(ub)[-40:],
                                     np.nonzero((ub > 2048) & (ub <= 8192))[0][:60]]))
    want = port.serial_rows(powerlaw, powerlaw, rows)
    assert rows_equal(powerlaw_product, want, rows)


def test_powerlaw_full_bound_sampled(port, powerlaw, powerlaw_product):
    rows = np.random.default_rng(8).choice(powerlaw.rows, 120, replace=False)
    c = powerlaw_product
    sub_rp = np.zeros(len(rows) + 1, np.int64)
    cols, vals = [], []
    for i, r in enumerate(rows):
        a0, a1 = c.row_ptr[r], c.row_ptr[r + 1]
        cols.append(c.col[a0:a1])
        vals.append(c.val[a0:a1])
        sub_rp[i + 1] = sub_rp[i] + a1 - a0
    sub = sg.Csr(len(rows), c.cols, sub_rp, np.concatenate(cols), np.concatenate(vals))
    rep = port.validate_full(powerlaw, powerlaw, sub, rows=rows)
    assert rep["passed"] and rep["rejected"] == 0 and rep["row_nnz_mismatches"] == 0
    assert rep["max_error_ratio"] <= 1.0


def test_powerlaw_power_of_two_scaling(engine, powerlaw, powerlaw_product):
    twice = engine.multiply(powerlaw.scaled(2.0), powerlaw)
    assert np.array_equal(twice.row_ptr, powerlaw_product.row_ptr)
    assert np.array_equal(twice.col, powerlaw_product.col)
    assert np.array_equal(twice.val, 2.0 * powerlaw_product.val)


@pytest.mark.parametrize("products", [2049, 4096, 4097, 8192, 20000])
@pytest.mark.parametrize("span", [(1 << 19) - 1, (1 << 20) - 1, (1 << 20)])
def test_packed_key_limits(engine, port, products, span):
    # one output row whose columns span exactly `span` + 1 values and whose
    # product count sits at a bin edge: the packed sort key uses all 32 bits
    rng = np.random.default_rng(products + span)
    ncols = span + 1
    k = 64
    blen = np.full(k, products // k)
    blen[: products % k] += 1
    brp = np.concatenate([[0], np.cumsum(blen)])
    bcol = rng.integers(0, ncols, size=int(brp[-1])).astype(np.int32)
    bcol[0], bcol[-1] = 0, span  # pin both ends of the range
    b = sg.Csr(k, ncols, brp, bcol, rng.uniform(-1, 1, size=int(brp[-1])))
    a = sg.Csr(2, k, np.array([0, k, 2 * k]), np.tile(np.arange(k, dtype=np.int32), 2), rng.uniform(-1, 1, 2 * k))
    got = engine.multiply(a, b)
    want = port.serial_spgemm(a, b)
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_powerlaw_exact_mode_full_validation(port, powerlaw):
    # the exact layout (symbolic pass, compacted output, global-slab heavy rows), every coordinate
    # checked on the GPU against the sequential sum: max |c - serial| = 0 means bit-identical
    with sg.Engine(0, mode="exact") as eng:
        da = powerlaw.to_device()
        c = eng.multiply(da, da, out="device")
        rep = eng.validate_full(da, da, c)
        c.free()
    assert rep["passed"] == 1 and rep["partial_passed"] == 1 and rep["max_abs_error"] == 0.0
    assert rep["reference_nnz"] == 583643070 and rep["support_mismatches"] == 0


def test_powerlaw_to_host_full_validation(engine, powerlaw):
    # the overlapped row-block path at full size (10 row blocks), checked on the GPU
    import torch
    p = engine.scalar_multiplication_count(powerlaw, powerlaw)
    rp = torch.empty(powerlaw.rows + 1, dtype=torch.int64, pin_memory=True)
    ci = torch.empty(p, dtype=torch.int32, pin_memory=True)
    va = torch.empty(p, dtype=torch.float64, pin_memory=True)
    nnz = engine.multiply_to_host(powerlaw, powerlaw, rp, ci, va)
    c = sg.Csr(powerlaw.rows, powerlaw.cols, rp.numpy(), ci.numpy()[:nnz], va.numpy()[:nnz])
    rep = engine.validate_full(powerlaw, powerlaw, c)
    assert rep["passed"] == 1 and rep["max_abs_error"] == 0.0 and rep["reference_nnz"] == nnz == 583643070
