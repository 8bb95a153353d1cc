"""The batched workload's own products (config 4's size distribution: square
products of 1,000-200,000 rows, 4-64 distinct uniform columns per row) through
the batched path -- every row of every product flattened into one work list of
(product << 32 | row) items, one launch per bin for all of them -- checked
against the oracle's serial product (spgemm_common.cpp:131-178): every row of
the smallest products, and a sample of rows, the heaviest included, of the
rest.  The same products through the serving loop must give the same bits."""
from __future__ import annotations

import numpy as np
import pytest

import spgemm_gb300 as sg
from helpers import csr_bits_equal, explain_diff

pytestmark = pytest.mark.gpu

COUNT = 48      # the first products of the batched workload's 512 (same seeds as bench.py)
FULL = 20       # the smallest ones are compared in full
SAMPLE = 64     # rows compared per remaining product


def batched_products():
    import bench
    return bench.make_workload("batched", count=COUNT)


def rows_of(c, rows):
    rp = np.asarray(c.row_ptr)
    parts = [(int(rp[r]), int(rp[r + 1])) for r in rows]
    out_rp = np.zeros(len(rows) + 1, dtype=np.int64)
    np.cumsum([e - s for s, e in parts], out=out_rp[1:])
    col = np.concatenate([np.asarray(c.col)[s:e] for s, e in parts])
    val = np.concatenate([np.asarray(c.val)[s:e] for s, e in parts])
    return sg.Csr(len(rows), c.cols, out_rp, col.astype(np.int32), val)


def test_batched_products_match_the_oracle(engine, port):
    pairs = batched_products()
    got = engine.multiply_batch(pairs)
    order = np.argsort([a.rows for a, _ in pairs])
    rng = np.random.default_rng(9)
    for rank, j in enumerate(order):
        a, b = pairs[j]
        c = got[j]
        if rank < FULL:
            want = port.serial_spgemm(a, b)
            assert csr_bits_equal(c, want), f"product {j}: " + explain_diff(c, want)
            continue
        ub = np.diff(b.row_ptr)[a.col]
        per_row = np.bincount(np.repeat(np.arange(a.rows), np.diff(a.row_ptr)), weights=ub, minlength=a.rows)
        rows = np.unique(np.concatenate([np.argsort(per_row)[-8:], rng.choice(a.rows, SAMPLE, replace=False)]))
        want = port.serial_rows(a, b, rows)
        assert csr_bits_equal(rows_of(c, rows), want), f"product {j}: " + explain_diff(rows_of(c, rows), want)


def test_served_products_equal_the_batched_ones(engine):
    pairs = batched_products()[:16]
    want = engine.multiply_batch(pairs)
    with sg.Server(0, lanes=2, max_batch=8, out="host") as srv:
        tickets = [srv.submit(a, b) for a, b in pairs]
        for t, w in zip(tickets, want):
            st, res, info = srv.poll(t)
            assert st == "SPG_OK", info
            got = res.download()
            assert csr_bits_equal(got, w), explain_diff(got, w)
