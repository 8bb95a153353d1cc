"""Multi-GPU row sharding, host side (CPU, gloo, world size 2): the cut of
A's rows by the prefix of their scalar products, the slices, and the gather of
the row blocks must rebuild, bit for bit, the product of one rank -- the
contract of the reference's partitionRows / distributeMatrix / gatherCsrMatrix
(src/common/spgemm_common.cpp:326-468).  Each rank's multiply here is the
oracle's serial product (the GPU multiply needs a GPU; the same code path takes
it as its callable on GPU hosts)."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PATHS = (str(ROOT), str(ROOT / "spgemm-hpc-thesis_gb300"), str(ROOT / "tests"))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case():
    from helpers import random_csr
    rng = np.random.default_rng(17)
    lens = rng.integers(0, 30, size=300)
    lens[50:60] = 0          # empty rows
    lens[120] = 200          # one heavy row
    a = random_csr(300, 250, lens, 3)
    b = random_csr(250, 280, rng.integers(0, 25, size=250), 4)
    return a, b


def test_partition_balances_products():
    import sharding
    from spgemm_gb300 import Csr
    a, b = _case()
    per_row = sharding.row_products(a, b)
    total = int(per_row.sum())
    prefix = np.concatenate([[0], np.cumsum(per_row)])
    for parts in (1, 2, 3, 7, 16):
        first = sharding.partition_rows(a, b, parts)
        assert first[0] == 0 and first[-1] == a.rows and np.all(np.diff(first) >= 0)
        for k in range(1, parts):
            # the first row whose preceding products reach floor(k * P / parts)
            target = total * k // parts
            assert prefix[first[k]] >= target and (first[k] == 0 or prefix[first[k] - 1] < target)
        loads = [int(per_row[first[k]:first[k + 1]].sum()) for k in range(parts)]
        assert sum(loads) == total and max(loads) <= total // parts + int(per_row.max())
    # no products at all: split by row count, as partitionRows does
    empty = Csr.from_arrays(10, 5, np.zeros(11, np.int64), [], [])
    bb = Csr.from_arrays(5, 5, np.zeros(6, np.int64), [], [])
    assert sharding.partition_rows(empty, bb, 3).tolist() == [0, 3, 6, 10]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    for p in PATHS:
        sys.path.insert(0, p)
    import torch.distributed as dist
    import sharding
    from oracle.oracle import Port
    dist.init_process_group("gloo", rank=rank, world_size=world)
    oracle = Port()
    a, b = _case()
    first, local, full = sharding.sharded_multiply(oracle.serial_spgemm, a, b, rank, world)
    same = None
    if rank == 0:
        want = oracle.serial_spgemm(a, b)
        same = (np.array_equal(full.row_ptr, want.row_ptr) and np.array_equal(full.col, want.col)
                and np.array_equal(full.val.view(np.uint64), want.val.view(np.uint64)))
    out.put((rank, first.tolist(), local.rows, same))
    dist.destroy_process_group()


def test_two_ranks_rebuild_the_product():
    pytest.importorskip("torch")
    from oracle import build as obuild
    obuild.build_oracle()
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, first0, rows0, same), (_, first1, rows1, _) = results
    assert first0 == first1 and rows0 + rows1 == 300 and rows0 == first0[1]
    assert same, "the gathered row blocks differ from the one-rank product"
