"""Rows above 8,192 scalar products in the upper-bound layout: a planner stages
each such row's products once, in product order, and cuts the row by column
range into pieces of at most 4,096 products, which run on the 4,096-product CTA
pipeline; a row with a bucket of more than 4,096 products keeps the global-slab
sort.  Every result must equal the serial reference product bit for bit
(spgemm_common.cpp:131-178), in batches and in the accumulate mode too
(matrix_blocks.cpp:152-200)."""
from __future__ import annotations

import numpy as np
import pytest

import spgemm_gb300 as sg
from helpers import csr_bits_equal, explain_diff, random_csr, row_sizes_for_bins

pytestmark = pytest.mark.gpu


def bucket_boundary_case(seed: int = 7):
    """B has 3,000 columns, so each planner bucket is one column; every B row
    holds column 5 and two other columns.  Output row 0 (12,288 products) gets
    exactly 4,096 products in column 5: one piece of exactly the piece capacity,
    summed as one run of 4,096 in product order.  Row 1 (12,291 products) gets
    4,097 there: unsplittable, the global-slab sort.  Row 2 is small."""
    rng = np.random.default_rng(seed)
    nb, ncols = 5000, 3000
    cols = np.empty((nb, 3), dtype=np.int64)
    cols[:, 0] = 5
    cols[:, 1:] = rng.integers(0, ncols, size=(nb, 2))
    for r in range(nb):
        rng.shuffle(cols[r])
    b = sg.Csr(nb, ncols, np.arange(nb + 1, dtype=np.int64) * 3, cols.reshape(-1).astype(np.int32),
               rng.uniform(-1, 1, size=3 * nb))
    rows = [rng.permutation(4096), rng.permutation(4097), rng.integers(0, nb, size=9)]
    rp = np.zeros(len(rows) + 1, dtype=np.int64)
    rp[1:] = np.cumsum([len(r) for r in rows])
    a = sg.Csr(len(rows), nb, rp, np.concatenate(rows).astype(np.int32), rng.uniform(-1, 1, size=int(rp[-1])))
    return a, b


@pytest.mark.parametrize("mode", ["upper_bound", "exact"])
def test_piece_capacity_boundary(port, mode):
    a, b = bucket_boundary_case()
    want = port.serial_spgemm(a, b)
    with sg.Engine(0, mode=mode) as eng:
        got = eng.multiply(a, b)
        t = eng.last_timings()
    assert t["bin_rows"]["b<=12K"] == 1 and t["bin_rows"]["b<=16K"] == 1
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_split_rows_in_a_batch(engine, port):
    # three products with rows of 8,193-30,000 products share one staging area
    pairs = [row_sizes_for_bins(s) for s in (11, 12, 13)]
    outs = engine.multiply_batch(pairs)
    for (a, b), got in zip(pairs, outs):
        want = port.serial_spgemm(a, b)
        assert csr_bits_equal(got, want), explain_diff(got, want)


def test_split_rows_with_an_addend(engine, port):
    # stages 2 and 3 of rows 0 and 1: the accumulated row (about 4,800 entries
    # after stage 1) followed by about 6,000 new products, so the addend
    # segment is part of the staged row
    rng = np.random.default_rng(3)
    stages = []
    for s in range(3):
        a = random_csr(4, 400, [300, 300, 20, 0], 30 + s, duplicates=False)
        b = random_csr(400, 20000, rng.integers(15, 26, size=400), 40 + s, duplicates=False)
        stages.append((a, b))
    got = engine.accumulate(4, 20000, stages)
    want = port.accumulate(4, 20000, stages)
    t = engine.last_timings()
    assert t["bin_rows"]["b<=12K"] + t["bin_rows"]["b<=16K"] >= 1
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_repeated_calls_reuse_the_scratch(engine, port):
    a, b = row_sizes_for_bins(21)
    want = port.serial_spgemm(a, b)
    for _ in range(3):
        got = engine.multiply(a, b)
        assert csr_bits_equal(got, want), explain_diff(got, want)
