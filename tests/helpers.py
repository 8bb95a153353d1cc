"""Seeded test inputs and comparison helpers (CPU only)."""
from __future__ import annotations

import numpy as np

from spgemm_gb300 import Csr


def random_csr(rows: int, cols: int, lengths, seed: int, *, unsorted: bool = True, duplicates: bool = True,
               zeros: bool = True, values: str = "uniform") -> Csr:
    """A CSR matrix whose row i has lengths[i] entries (an int gives every row
    that length).  With `unsorted`/`duplicates`/`zeros` the rows keep file-order
    columns, repeated columns and explicit zeros, as the reference's Matrix
    Market reader produces them (matrix_market.cpp:129-143).  values:
    "uniform" U[-1, 1), "dyadic" small multiples of 2^-3 (exact sums, frequent
    cancellation), "int" integers in [-3, 3]."""
    rng = np.random.default_rng(seed)
    lens = np.full(rows, lengths, dtype=np.int64) if np.isscalar(lengths) else np.asarray(lengths, dtype=np.int64)
    if cols == 0:
        lens[:] = 0
    rp = np.zeros(rows + 1, dtype=np.int64)
    np.cumsum(lens, out=rp[1:])
    nnz = int(rp[-1])
    if duplicates:
        col = rng.integers(0, max(cols, 1), size=nnz, dtype=np.int64)
    else:
        col = np.empty(nnz, dtype=np.int64)
        for r in range(rows):
            k = int(lens[r])
            col[rp[r]:rp[r + 1]] = rng.choice(cols, size=min(k, cols), replace=False) if k else []
    if not unsorted:
        for r in range(rows):
            col[rp[r]:rp[r + 1]] = np.sort(col[rp[r]:rp[r + 1]])
    if values == "uniform":
        val = rng.uniform(-1.0, 1.0, size=nnz)
    elif values == "dyadic":
        val = rng.integers(-4, 5, size=nnz).astype(np.float64) * 0.125
    else:
        val = rng.integers(-3, 4, size=nnz).astype(np.float64)
    if zeros and nnz:
        val[rng.random(nnz) < 0.05] = 0.0
    return Csr(rows, cols, rp, col.astype(np.int32), val)


def csr_bits_equal(x, y) -> bool:
    return (int(x.rows) == int(y.rows) and int(x.cols) == int(y.cols)
            and np.array_equal(np.asarray(x.row_ptr), np.asarray(y.row_ptr))
            and np.array_equal(np.asarray(x.col), np.asarray(y.col))
            and np.array_equal(np.asarray(x.val, dtype=np.float64).view(np.uint64),
                               np.asarray(y.val, dtype=np.float64).view(np.uint64)))


def explain_diff(x, y) -> str:
    if (x.rows, x.cols) != (y.rows, y.cols):
        return f"shape {(x.rows, x.cols)} vs {(y.rows, y.cols)}"
    rx, ry = np.asarray(x.row_ptr), np.asarray(y.row_ptr)
    bad = np.nonzero(np.diff(rx) != np.diff(ry))[0]
    if len(bad):
        r = int(bad[0])
        return (f"{len(bad)} rows differ in count; first row {r}: {rx[r+1]-rx[r]} vs {ry[r+1]-ry[r]}; "
                f"cols {x.col[rx[r]:rx[r+1]][:8]} vs {y.col[ry[r]:ry[r+1]][:8]}")
    cbad = np.nonzero(np.asarray(x.col) != np.asarray(y.col))[0]
    if len(cbad):
        return f"{len(cbad)} columns differ, first at {cbad[0]}"
    vx = np.asarray(x.val).view(np.uint64)
    vy = np.asarray(y.val).view(np.uint64)
    vbad = np.nonzero(vx != vy)[0]
    if len(vbad):
        i = int(vbad[0])
        return f"{len(vbad)} values differ, first at {i}: {x.val[i]!r} vs {y.val[i]!r}"
    return "equal"


def row_sizes_for_bins(seed: int):
    """(A, B) whose rows cover every product-count bin of the engine, the
    heavy (> 16384 products) one included."""
    rng = np.random.default_rng(seed)
    targets = [0, 1, 7, 32, 33, 64, 65, 96, 97, 128, 129, 192, 193, 256, 257, 384, 385, 512, 513, 768, 769, 1024,
               1025, 1536, 1537, 2048, 2049, 3072, 3073, 4096, 4097, 6144, 6145, 8192, 8193, 12288, 12289, 16384,
               16385, 30000]
    lens = rng.integers(0, 41, size=4000)
    lens[:100] = 1  # rows of one entry make every exact product count reachable
    b = random_csr(4000, 3000, lens, seed + 1)
    bl = np.diff(b.row_ptr)
    rows_cols = []
    for t in targets:
        cols, acc = [], 0
        while True:
            k = int(rng.integers(100, 4000))
            if acc + bl[k] > t:
                break
            cols.append(k)
            acc += int(bl[k])
        while acc < t:
            cols.append(int(rng.integers(0, 100)))
            acc += 1
        rng.shuffle(cols)
        rows_cols.append(cols)
    rp = np.zeros(len(targets) + 1, dtype=np.int64)
    rp[1:] = np.cumsum([len(c) for c in rows_cols])
    col = np.array([c for cs in rows_cols for c in cs], dtype=np.int32)
    val = rng.uniform(-1, 1, size=len(col))
    a = Csr(len(targets), 4000, rp, col, val)
    return a, b
