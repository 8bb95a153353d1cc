"""Row sharding on the GPU: spg_partition_rows (device row work and scan) cuts
A's rows exactly where the host-side partition does, and the engine's row
blocks, appended in order, equal the one-call product bit for bit (the blocks
run one after the other on one GPU here; on G GPUs each rank runs one)."""
from __future__ import annotations

import numpy as np
import pytest

import sharding
from helpers import csr_bits_equal, explain_diff, random_csr
from spgemm_gb300 import synth_powerlaw

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("where", ["host", "device"])
def test_device_partition_equals_host_partition(engine, where):
    a = synth_powerlaw(65536, 24.0, 1.2, 20000, 2048, 0.7, seed=5)
    for parts in (1, 2, 4, 8, 152):
        want = sharding.partition_rows(a, a, parts)
        op = a if where == "host" else a.to_device()
        got = engine.partition_rows(op, op, parts)
        assert np.array_equal(got, want), (parts, got[:8], want[:8])


def test_row_blocks_rebuild_the_product(engine, port):
    rng = np.random.default_rng(3)
    a = random_csr(2000, 1500, rng.integers(0, 40, size=2000), 7)
    b = random_csr(1500, 1800, rng.integers(0, 30, size=1500), 8)
    first = engine.partition_rows(a, b, 4)
    blocks = [engine.multiply(sharding.slice_rows(a, int(first[k]), int(first[k + 1] - first[k])), b)
              for k in range(4)]
    got = sharding.append_blocks(blocks, a.rows, b.cols)
    want = port.serial_spgemm(a, b)
    assert csr_bits_equal(got, want), explain_diff(got, want)
