"""GPU parity: the CUDA engine, called through the C ABI, against the CPU oracle.

The bar is bit-exactness: row offsets, columns and the 64-bit patterns of the
values must equal the serial reference product (spgemm_common.cpp:131-178),
because the engine sums every coordinate in the reference's order with the
reference's roundings.  Inputs cover the reference tests' edge cases: unsorted
rows, duplicate columns, explicit zeros, empty rows and columns, exact
cancellation, non-finite values, overflow and underflow, rectangular shapes,
and every row-size bin of the engine including the heavy one.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import csr_bits_equal, explain_diff, random_csr, row_sizes_for_bins
from spgemm_gb300 import Csr, SpgError

pytestmark = pytest.mark.gpu


def check(engine, port, a, b):
    got = engine.multiply(a, b)
    want = port.serial_spgemm(a, b)
    assert csr_bits_equal(got, want), explain_diff(got, want)
    return got


@pytest.mark.parametrize("seed", range(12))
def test_random_small(engine, port, seed):
    rng = np.random.default_rng(seed)
    m, k, n = (int(x) for x in rng.integers(1, 60, size=3))
    a = random_csr(m, k, rng.integers(0, 2 * k + 2, size=m), seed)
    b = random_csr(k, n, rng.integers(0, 2 * n + 2, size=k), seed + 100)
    check(engine, port, a, b)


@pytest.mark.parametrize("values", ["dyadic", "int"])
def test_cancellation_heavy_inputs(engine, port, values):
    # small integer / dyadic values cancel exactly and often
    a = random_csr(200, 50, 30, 7, values=values)
    b = random_csr(50, 40, 25, 8, values=values)
    c = check(engine, port, a, b)
    assert np.all(c.val != 0.0)


@pytest.mark.parametrize("seed", [1, 2])
def test_every_bin(engine, port, seed):
    a, b = row_sizes_for_bins(seed)
    check(engine, port, a, b)
    t = engine.last_timings()
    from spgemm_gb300 import BIN_NAMES
    assert all(t["bin_rows"][name] >= 1 for name in BIN_NAMES), t["bin_rows"]


def column_window_case(width: int, seed: int):
    """(A, B) whose every output row spans exactly 2**width columns (the window
    [base, base + 2**width - 1], both ends in every B row), with rows of 0, 40,
    200, 500, 1,200, 3,000 and 15,000 scalar products (warp-row bins, CTA
    bins with shared and global value slabs, the 16K bin)."""
    rng = np.random.default_rng(seed)
    base = 1000
    lo, hi = base, base + (1 << width) - 1
    inner, blen = 200, 20
    cols = rng.integers(lo, hi + 1, size=(inner, blen), dtype=np.int64)
    cols[:, 0], cols[:, 1] = lo, hi
    for r in range(inner):
        rng.shuffle(cols[r])
    b = Csr(inner, hi + 7, np.arange(inner + 1, dtype=np.int64) * blen, cols.reshape(-1).astype(np.int32),
            rng.uniform(-1, 1, size=inner * blen))
    counts = [0, 2, 10, 25, 60, 150, 750]  # A entries per row: products = 20 x count
    rp = np.zeros(len(counts) + 1, dtype=np.int64)
    rp[1:] = np.cumsum(counts)
    a = Csr(len(counts), inner, rp, rng.integers(0, inner, size=int(rp[-1])).astype(np.int32),
            rng.uniform(-1, 1, size=int(rp[-1])))
    return a, b


def test_repeated_columns_next_to_wide_rows(engine, port):
    # Rows whose products fall on three columns (a column repeated more than 64
    # times makes the bucket sort hand the row to the radix sort) interleaved
    # with rows of wide column ranges, in every bin from 100 to 6,000 products:
    # in one launch some teams of a kernel take the radix fallback and others do
    # not, which must not disturb one another's results or the stored count.
    rng = np.random.default_rng(11)
    nb = 2000
    b_cols = np.where(np.arange(nb)[:, None] < nb // 2, rng.integers(0, 3, size=(nb, 16)),
                      rng.integers(0, 3000, size=(nb, 16))).astype(np.int32)
    b = Csr(nb, 3000, np.arange(0, 16 * nb + 1, 16, dtype=np.int64), b_cols.ravel(),
            rng.uniform(-1, 1, size=16 * nb))
    rows = []
    for t in (100, 200, 240, 300, 450, 700, 1000, 1500, 3000, 6000):
        for r in range(64):
            lo = 0 if r % 2 == 0 else nb // 2
            rows.append(rng.integers(lo, lo + nb // 2, size=t // 16))
    rp = np.zeros(len(rows) + 1, dtype=np.int64)
    rp[1:] = np.cumsum([len(x) for x in rows])
    a = Csr(len(rows), nb, rp, np.concatenate(rows).astype(np.int32), rng.uniform(-1, 1, size=int(rp[-1])))
    check(engine, port, a, b)


@pytest.mark.parametrize("width", [0, 1, 3, 4, 5, 8, 9, 12, 13, 16, 17, 19, 20, 21, 24, 25])
def test_column_range_widths(engine, port, width):
    # The radix sort takes 8-bit passes and a last pass of at most 4 bits, over
    # the bits of max(col) - min(col) only; keys pack (column, sequence) into
    # 32 bits unless the width and the sequence bits exceed that (widths >= 19
    # in the 16K bin, >= 21 in the 3K bin, >= 25 in the warp bins).
    a, b = column_window_case(width, 40 + width)
    check(engine, port, a, b)


def test_known_answer(engine):
    # spgemm_serial_smoke.cpp:65-67
    a = Csr.from_arrays(2, 3, [0, 2, 3], [0, 2, 1], [1.0, 2.0, 3.0])
    b = Csr.from_arrays(3, 2, [0, 1, 2, 3], [1, 0, 1], [4.0, 5.0, 6.0])
    c = engine.multiply(a, b)
    assert c.row_ptr.tolist() == [0, 1, 2] and c.col.tolist() == [1, 0] and c.val.tolist() == [16.0, 15.0]
    assert engine.scalar_multiplication_count(a, b) == 3


def test_cancellation_and_empty_row(engine):
    # spgemm_validation_smoke.cpp:153-155
    a = Csr.from_arrays(3, 2, [0, 2, 2, 3], [0, 1, 1], [1, 1, 2])
    b = Csr.from_arrays(2, 3, [0, 2, 4], [0, 1, 0, 2], [1, 2, -1, 3])
    c = engine.multiply(a, b)
    assert c.row_ptr.tolist() == [0, 2, 2, 4]
    assert c.col.tolist() == [1, 2, 0, 2] and c.val.tolist() == [2, 3, -2, 6]


def test_summation_order(engine, port):
    # partial_reference_test.cpp:151-157: {1e16, -1e16, 1} keeps 1; {1e16, 1, -1e16} cancels
    a = Csr.from_arrays(1, 1, [0, 1], [0], [1.0])
    b1 = Csr.from_arrays(1, 1, [0, 3], [0, 0, 0], [1e16, -1e16, 1.0])
    b2 = Csr.from_arrays(1, 1, [0, 3], [0, 0, 0], [1e16, 1.0, -1e16])
    assert engine.multiply(a, b1).val.tolist() == [1.0]
    assert engine.multiply(a, b2).nnz == 0
    # spgemm_full_streaming.cpp:58-62: serial 1 + 2^-55 - 1 == 0
    tiny = 2.0 ** -55
    a3 = Csr.from_arrays(1, 3, [0, 3], [0, 1, 2], [1, 1, 1])
    b3 = Csr.from_arrays(3, 1, [0, 1, 2, 3], [0, 0, 0], [1, tiny, -1])
    assert engine.multiply(a3, b3).nnz == 0


def test_nonfinite_overflow_underflow(engine, port):
    huge = Csr.from_arrays(1, 1, [0, 1], [0], [1e200])
    c = engine.multiply(huge, huge)
    assert c.nnz == 1 and np.isinf(c.val[0])
    tiny = Csr.from_arrays(1, 1, [0, 1], [0], [1e-200])
    assert engine.multiply(tiny, tiny).nnz == 0
    sub = Csr.from_arrays(1, 1, [0, 1], [0], [np.finfo(np.float64).smallest_subnormal])
    unit = Csr.from_arrays(1, 1, [0, 1], [0], [1.0])
    assert engine.multiply(sub, unit).val.view(np.uint64).tolist() == [1]
    for v in (np.nan, np.inf, -np.inf):
        a = random_csr(20, 10, 6, 3)
        a.val[3] = v
        b = random_csr(10, 12, 5, 4)
        got, want = engine.multiply(a, b), port.serial_spgemm(a, b)
        assert np.array_equal(got.row_ptr, want.row_ptr) and np.array_equal(got.col, want.col)
        assert np.array_equal(np.isnan(got.val), np.isnan(want.val))
        fin = ~np.isnan(want.val)
        assert np.array_equal(got.val[fin].view(np.uint64), want.val[fin].view(np.uint64))


@pytest.mark.parametrize("shape", [(7, 9, 5), (1, 1, 1), (0, 3, 2), (3, 0, 4), (3, 4, 0), (19, 11, 13)])
def test_shape_sweep(engine, port, shape):
    # the shapes of trident_correctness.cpp:207-210
    m, k, n = shape
    a = random_csr(m, k, min(k, 4) if k else 0, 11)
    b = random_csr(k, n, min(n, 3) if n else 0, 12)
    check(engine, port, a, b)


def test_device_operands_and_results(engine, port):
    a = random_csr(300, 200, 12, 21)
    b = random_csr(200, 250, 9, 22)
    want = port.serial_spgemm(a, b)
    r = engine.multiply(a.to_device(), b.to_device(), out="device")
    got = r.download()
    r.free()
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_errors(engine):
    a = Csr.from_arrays(2, 3, [0, 1, 2], [0, 2], [1.0, 1.0])
    with pytest.raises(SpgError) as e:
        engine.multiply(a, Csr.from_arrays(2, 2, [0, 1, 2], [0, 1], [1.0, 1.0]))
    assert e.value.name == "SPG_INVALID_ARGUMENT"
    bad = Csr.from_arrays(2, 3, [0, 1, 2], [0, 7], [1.0, 1.0])
    with pytest.raises(SpgError) as e:
        engine.multiply(bad, Csr.from_arrays(3, 2, [0, 1, 2, 3], [0, 1, 0], [1.0, 1.0, 1.0]))
    assert e.value.name == "SPG_OUT_OF_RANGE_COLUMN"
    badb = Csr.from_arrays(3, 2, [0, 1, 2, 3], [5, 1, 0], [1.0, 1.0, 1.0])
    with pytest.raises(SpgError) as e:
        engine.multiply(a, badb)
    assert e.value.name == "SPG_INVALID_ARGUMENT"
    # the handle stays usable after errors
    ok = engine.multiply(a, Csr.from_arrays(3, 2, [0, 1, 2, 3], [0, 1, 0], [1.0, 1.0, 1.0]))
    assert ok.nnz == 2


def test_accumulate_matches_local_accumulator(engine, port):
    # trident_accumulator_memory.cpp:40-60: three stages with cross-stage cancellation
    a = Csr.from_arrays(3, 2, [0, 3, 3, 4], [1, 0, 1, 0], [2.0, 1.0, -1.0, 3.0])
    b = Csr.from_arrays(2, 4, [0, 3, 5], [3, 1, 3, 0, 1], [2.0, 4.0, -1.0, 5.0, -4.0])
    a2, a3 = a.scaled(-1.0), a.scaled(0.5)
    got = engine.accumulate(3, 4, [(a, b), (a2, b), (a3, b)])
    want = port.accumulate(3, 4, [(a, b), (a2, b), (a3, b)])
    assert csr_bits_equal(got, want), explain_diff(got, want)
    assert got.row_ptr[1] == got.row_ptr[2]


@pytest.mark.parametrize("seed", [3, 4])
def test_accumulate_random(engine, port, seed):
    rng = np.random.default_rng(seed)
    stages = []
    for s in range(4):
        k = int(rng.integers(1, 30))
        stages.append((random_csr(40, k, rng.integers(0, 10, size=40), seed * 10 + s),
                       random_csr(k, 35, rng.integers(0, 12, size=k), seed * 10 + s + 5, values="dyadic")))
    got = engine.accumulate(40, 35, stages)
    want = port.accumulate(40, 35, stages)
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_accumulate_dense_outer_product(engine, port):
    # trident_accumulator_memory.cpp:12-38 with n = 300: two identical stages
    n = 300
    a = Csr.from_arrays(n, 1, np.arange(n + 1), np.zeros(n), np.ones(n))
    b = Csr.from_arrays(1, n, [0, n], np.arange(n), np.arange(1, n + 1, dtype=np.float64))
    c = engine.accumulate(n, n, [(a, b), (a, b)])
    assert c.nnz == n * n
    assert np.array_equal(c.val.reshape(n, n), np.tile(2.0 * np.arange(1, n + 1), (n, 1)))


def test_accumulate_shape_errors(engine):
    a = Csr.from_arrays(2, 2, [0, 1, 2], [0, 1], [1.0, 1.0])
    with pytest.raises(SpgError) as e:
        engine.accumulate(3, 2, [(a, a)])
    assert e.value.name == "SPG_INVALID_ARGUMENT"


def test_batch_equals_single(engine, port):
    rng = np.random.default_rng(5)
    pairs = []
    for i in range(9):
        m, k, n = (int(x) for x in rng.integers(0, 80, size=3))
        pairs.append((random_csr(m, k, rng.integers(0, 3 * max(k, 1), size=m) if k else 0, 50 + i),
                      random_csr(k, n, rng.integers(0, 3 * max(n, 1), size=k) if n else 0, 80 + i)))
    outs = engine.multiply_batch(pairs)
    for (a, b), got in zip(pairs, outs):
        want = port.serial_spgemm(a, b)
        assert csr_bits_equal(got, want), explain_diff(got, want)


@pytest.mark.parametrize("mode", ["exact", "upper_bound"])
def test_output_modes(port, mode):
    import spgemm_gb300 as sg
    with sg.Engine(0, mode=mode) as eng:
        for seed in (1, 2):
            a, b = row_sizes_for_bins(seed)
            check(eng, port, a, b)
        a = random_csr(300, 40, 25, 9, values="int")
        b = random_csr(40, 50, 20, 10, values="int")
        check(eng, port, a, b)  # many exact cancellations: rows shrink after summation
        acc = eng.accumulate(40, 35, [(random_csr(40, 9, 5, 11), random_csr(9, 35, 6, 12, values="dyadic"))] * 3)
        want = port.accumulate(40, 35, [(random_csr(40, 9, 5, 11), random_csr(9, 35, 6, 12, values="dyadic"))] * 3)
        assert csr_bits_equal(acc, want), explain_diff(acc, want)


def test_budget_exceeded(port):
    import spgemm_gb300 as sg
    a = random_csr(2000, 2000, 30, 13)
    with sg.Engine(0, hbm_budget_bytes=64 << 10) as eng:
        with pytest.raises(SpgError) as e:
            eng.multiply(a, a)
        assert e.value.name == "SPG_BUDGET_EXCEEDED"
        small = random_csr(4, 4, 2, 14)
        check(eng, port, small, small)


def test_repeatable(engine):
    a = random_csr(500, 400, 30, 31)
    b = random_csr(400, 450, 25, 32)
    c1, c2 = engine.multiply(a, b), engine.multiply(a, b)
    assert csr_bits_equal(c1, c2)
