"""bench.py with several ranks (CPU, gloo, world size 2): the ranks' wall
times reduce to the slowest rank and their products to the job total, and the
reference arm runs on rank 0 only.  No data-path collective exists: each rank
multiplies its own block of rows."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, local = bench.dist_init()
    bench.barrier(w)
    slowest = bench.all_max(10.0 + r, w)
    total = bench.all_sum(100.0 * (r + 1), w)

    class Args:
        workload, rows, warmup, steps, reference_step_seconds = "uniform", 0, 3, 1, 1.0

    returned = bench.run_reference_arm(Args(), r, w) if r != 0 else None  # ranks != 0 leave at once
    out.put((r, w, local, slowest, total, returned))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_ranks_reduce_and_split_roles():
    torch = pytest.importorskip("torch")
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
    assert [r[0] for r in results] == [0, 1] and all(r[1] == 2 for r in results)
    assert all(r[3] == 11.0 for r in results)      # max over ranks
    assert all(r[4] == 300.0 for r in results)     # sum over ranks
    assert results[1][5] is None                   # the reference arm returned on rank 1 without work
