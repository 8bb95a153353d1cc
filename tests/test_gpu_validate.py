"""GPU tests of the validator (spg_validate_full): the reference's Full and
Partial modes (spgemm_common.cpp:541-572, 720-851) recomputed on the GPU must
agree with the CPU oracle's restatement of them, catch mistakes planted in C,
and pass the engine's full-size products."""
from __future__ import annotations

import math

import numpy as np
import pytest

from helpers import random_csr, row_sizes_for_bins
from spgemm_gb300 import Csr, synth_powerlaw

pytestmark = pytest.mark.gpu

EXACT = ("passed", "matrices_ok", "rejected", "row_nnz_mismatches", "support_mismatches", "reference_nnz",
         "checked_coordinates")


def agree(gpu: dict, cpu: dict):
    for k in EXACT:
        assert int(gpu[k]) == int(cpu[k]), (k, gpu, cpu)
    assert gpu["max_abs_error"] == cpu["max_abs_error"]
    # the reference sums differ in precision (double-double here, long double in the oracle)
    assert math.isclose(gpu["max_error_ratio"], cpu["max_error_ratio"], rel_tol=0.05, abs_tol=1e-12)
    assert math.isclose(gpu["max_rel_error"], cpu["max_rel_error"], rel_tol=1e-3, abs_tol=1e-30)
    if cpu["median_rel_error"] > 0:
        assert 0.9 < gpu["median_rel_error"] / cpu["median_rel_error"] < 1.1


@pytest.mark.parametrize("seed", range(4))
def test_agrees_with_oracle_on_engine_results(engine, port, seed):
    rng = np.random.default_rng(seed)
    m, k, n = (int(x) for x in rng.integers(20, 400, size=3))
    a = random_csr(m, k, rng.integers(0, 30, size=m), seed, zeros=False)
    b = random_csr(k, n, rng.integers(0, 30, size=k), seed + 7, zeros=False)
    c = engine.multiply(a, b)
    gpu = engine.validate_full(a, b, c)
    cpu = port.validate_full(a, b, c)
    assert gpu["passed"] == 1 and gpu["partial_passed"] == 1
    agree(gpu, cpu)


def test_every_bin_and_heavy_rows(engine, port):
    a, b = row_sizes_for_bins(2)
    c = engine.multiply(a, b)
    gpu = engine.validate_full(a, b, c)
    assert gpu["passed"] == 1 and gpu["max_abs_error"] == 0.0
    agree(gpu, port.validate_full(a, b, c))


@pytest.mark.parametrize("mistake", ["value", "drop", "extra", "order"])
def test_planted_mistakes_are_caught(engine, port, mistake):
    a = random_csr(120, 80, 9, 3, zeros=False)
    b = random_csr(80, 90, 7, 4, zeros=False)
    c = engine.multiply(a, b)
    rp, col, val = c.row_ptr.copy(), c.col.copy(), c.val.copy()
    row = int(np.argmax(np.diff(rp)))  # a row with several entries
    p0 = int(rp[row])
    if mistake == "value":
        val[p0] += 1.0
    elif mistake == "drop":
        col = np.delete(col, p0)
        val = np.delete(val, p0)
        rp[row + 1:] -= 1
    elif mistake == "extra":  # an entry at a column the product does not have
        present = set(col[rp[row]:rp[row + 1]].tolist())
        free = next(x for x in range(90) if x not in present)
        ins = int(np.searchsorted(col[rp[row]:rp[row + 1]], free)) + p0
        col = np.insert(col, ins, free)
        val = np.insert(val, ins, 0.5)
        rp[row + 1:] += 1
    else:  # two columns swapped: not sorted any more
        col[p0], col[p0 + 1] = col[p0 + 1], col[p0]
    bad = Csr(c.rows, c.cols, rp, col, val)
    gpu = engine.validate_full(a, b, bad)
    cpu = port.validate_full(a, b, bad)
    assert gpu["passed"] == 0
    agree(gpu, cpu)
    if mistake in ("drop", "extra"):
        assert gpu["row_nnz_mismatches"] == 1 and gpu["partial_passed"] == 0
    if mistake == "order":
        assert gpu["matrices_ok"] == 0


def test_non_finite_operands(engine, port):
    a = random_csr(30, 20, 5, 1)
    b = random_csr(20, 25, 5, 2)
    c = engine.multiply(a, b)
    a.val[2] = np.inf
    gpu = engine.validate_full(a, b, c)
    assert gpu["matrices_ok"] == 0 and gpu["passed"] == 0
    assert gpu["matrices_ok"] == port.validate_full(a, b, c)["matrices_ok"]


def test_full_size_powerlaw_passes(engine):
    # the bench's skewed workload: every coordinate of 583 M checked on the GPU
    a = synth_powerlaw(1 << 20, 24.0, 1.2, 20000, 2048, 0.7, seed=1)
    da = a.to_device()
    c = engine.multiply(da, da, out="device")
    rep = engine.validate_full(da, da, c)
    c.free()
    assert rep["matrices_ok"] == 1 and rep["passed"] == 1 and rep["partial_passed"] == 1
    assert rep["reference_nnz"] == 583643070 and rep["max_abs_error"] == 0.0
    assert rep["max_error_ratio"] < 1.0
