"""Single-node multi-GPU row sharding of one product (one process per GPU).

The reference distributes its multiply by output rows over MPI ranks:
``partitionRows`` cuts A's rows into equal counts
(src/common/spgemm_common.cpp:326-337), ``distributeMatrix`` sends each rank
its slice (``sliceRows``, :367-381, :383-424), every rank multiplies its rows,
fetching remote B rows through a halo exchange (src/baselines/
spgemm_exchange.cpp:91-256), and ``gatherCsrMatrix`` appends the row blocks on
rank 0 (:432-468).

Here every GPU holds all of B (replicated once: no exchange during the
multiply), the rows are cut by the prefix of their scalar products so that
each GPU gets about P / G products (``partition_rows``; the engine's
``spg_partition_rows`` computes the same cut on the device), each rank
multiplies its row block on its own GPU, and ``gather_csr`` appends the blocks
on one rank over ``torch.distributed`` point-to-point messages (the only
collective step, after the multiply, and optional).  The per-rank multiply is
a callable, so the partition, slicing and reassembly run unchanged with any
multiply.
"""
from __future__ import annotations

from typing import Callable

import numpy as np

from spgemm_gb300 import Csr


def row_products(a: Csr, b: Csr) -> np.ndarray:
    """Scalar products of every row of A * B (scalarMultiplicationCount per row,
    spgemm_common.cpp:474-487)."""
    per_entry = np.diff(np.asarray(b.row_ptr))[np.asarray(a.col)] if a.nnz else np.zeros(0, np.int64)
    rows_of = np.repeat(np.arange(a.rows), np.diff(np.asarray(a.row_ptr)))
    return np.bincount(rows_of, weights=per_entry, minlength=a.rows).astype(np.int64)


def partition_rows(a: Csr, b: Csr, parts: int) -> np.ndarray:
    """first_row[0..parts]: block k holds rows [first_row[k], first_row[k+1]),
    the first row whose preceding products reach floor(k * P / parts); by row
    count when there are no products (the reference's split)."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    prefix = np.zeros(a.rows + 1, dtype=np.int64)
    np.cumsum(row_products(a, b), out=prefix[1:])
    total = int(prefix[-1])
    first = np.empty(parts + 1, dtype=np.int64)
    for k in range(parts + 1):
        if k == 0:
            first[k] = 0
        elif k == parts:
            first[k] = a.rows
        elif total == 0:
            first[k] = a.rows * k // parts
        else:
            first[k] = int(np.searchsorted(prefix, (total * k) // parts, side="left"))
    return first.astype(np.int32)


def slice_rows(a: Csr, first: int, count: int) -> Csr:
    """Rows [first, first + count) of A with offsets restarting at zero (sliceRows)."""
    rp = np.asarray(a.row_ptr)[first:first + count + 1]
    lo, hi = int(rp[0]), int(rp[-1])
    return Csr(count, a.cols, rp - lo, np.asarray(a.col)[lo:hi], np.asarray(a.val)[lo:hi])


def append_blocks(blocks: list[Csr], rows: int, cols: int) -> Csr:
    """C from its row blocks in rank order (appendCsrBlock of gatherCsrMatrix)."""
    rp = np.zeros(rows + 1, dtype=np.int64)
    at, off = 0, 0
    for blk in blocks:
        brp = np.asarray(blk.row_ptr)
        rp[at + 1:at + blk.rows + 1] = brp[1:] + off
        at += blk.rows
        off += int(brp[-1])
    if at != rows:
        raise ValueError(f"row blocks cover {at} rows, expected {rows}")
    col = np.concatenate([np.asarray(b.col) for b in blocks]) if blocks else np.zeros(0, np.int32)
    val = np.concatenate([np.asarray(b.val) for b in blocks]) if blocks else np.zeros(0, np.float64)
    return Csr(rows, cols, rp, col.astype(np.int32), val.astype(np.float64))


def gather_csr(local: Csr, rank: int, world: int, rows: int, cols: int, dst: int = 0, group=None,
               device: str = "cpu") -> Csr | None:
    """Row blocks of every rank appended on rank `dst` (None elsewhere), over
    torch.distributed send/recv: a header (rows, nnz), then the offsets, columns
    and values -- the messages of gatherCsrMatrix.  `device` is where the
    message tensors live ("cuda" for NCCL)."""
    import torch
    import torch.distributed as dist

    def t(x, dtype):
        return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype).to(device)

    if rank != dst:
        nnz = int(np.asarray(local.row_ptr)[-1])
        dist.send(t([local.rows, nnz], torch.int64), dst, group=group)
        dist.send(t(local.row_ptr, torch.int64), dst, group=group)
        if nnz:
            dist.send(t(local.col, torch.int32), dst, group=group)
            dist.send(t(local.val, torch.float64), dst, group=group)
        return None
    blocks = []
    for peer in range(world):
        if peer == rank:
            blocks.append(local)
            continue
        hdr = torch.empty(2, dtype=torch.int64, device=device)
        dist.recv(hdr, peer, group=group)
        prow, pnnz = int(hdr[0]), int(hdr[1])
        rp = torch.empty(prow + 1, dtype=torch.int64, device=device)
        dist.recv(rp, peer, group=group)
        col = torch.empty(pnnz, dtype=torch.int32, device=device)
        val = torch.empty(pnnz, dtype=torch.float64, device=device)
        if pnnz:
            dist.recv(col, peer, group=group)
            dist.recv(val, peer, group=group)
        blocks.append(Csr(prow, cols, rp.cpu().numpy(), col.cpu().numpy(), val.cpu().numpy()))
    return append_blocks(blocks, rows, cols)


def sharded_multiply(multiply: Callable[[Csr, Csr], Csr], a: Csr, b: Csr, rank: int, world: int,
                     gather: bool = True, dst: int = 0, group=None, device: str = "cpu",
                     first_row: np.ndarray | None = None):
    """C = A * B over `world` ranks: this rank multiplies its row block of A
    (partition_rows, or the given cut) against all of B with `multiply`.
    Returns (first_row, local block, C on rank `dst` when gathering else None)."""
    first = partition_rows(a, b, world) if first_row is None else np.asarray(first_row)
    r0, r1 = int(first[rank]), int(first[rank + 1])
    local = multiply(slice_rows(a, r0, r1 - r0), b)
    if world == 1:
        return first, local, local
    full = gather_csr(local, rank, world, a.rows, b.cols, dst, group, device) if gather else None
    return first, local, full
