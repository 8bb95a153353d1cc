"""The Matrix Market reader with device output (spg_read_matrix_market with
SPG_DEVICE): the device arrays must equal the host reader's, which the CPU
tests pin to the reference's readMatrixMarket (matrix_market.cpp:28-145), and
they must feed the multiply directly."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import csr_bits_equal, explain_diff
from spgemm_gb300 import Csr, read_matrix_market

pytestmark = pytest.mark.gpu


def to_host(d) -> Csr:
    return Csr(d.rows, d.cols, d.row_ptr.cpu().numpy(), d.col.cpu().numpy(), d.val.cpu().numpy())


@pytest.mark.parametrize("text", [
    "%%MatrixMarket matrix coordinate real general\n% c\n3 4 5\n1 1 1.5\n3 4 -2\n1 2 3e2\n1 1 0.25\n2 3 4D-1\n",
    "%%MatrixMarket matrix coordinate real symmetric\n3 3 4\n1 1 2\n3 1 -1\n2 1 0.5\n3 3 7\n",
    "%%MatrixMarket matrix coordinate pattern general\n2 3 3\n1 3\n2 1\n1 3\n",
    "%%MatrixMarket matrix coordinate real general\n5 6 0\n",
])
def test_device_output_equals_host_output(tmp_path, text):
    p = tmp_path / "m.mtx"
    p.write_bytes(text.encode())
    want = read_matrix_market(p)
    got = to_host(read_matrix_market(p, out="device"))
    assert csr_bits_equal(got, want), explain_diff(got, want)


def test_device_read_feeds_the_multiply(tmp_path, engine, port):
    rng = np.random.default_rng(11)
    n, nnz = 400, 3000
    rows = rng.integers(1, n + 1, size=nnz)
    cols = rng.integers(1, n + 1, size=nnz)
    vals = rng.integers(-4, 5, size=nnz) * 0.25
    lines = [f"{int(r)} {int(c)} {float(v)!r}" for r, c, v in zip(rows, cols, vals)]
    p = tmp_path / "big.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n" + f"{n} {n} {nnz}\n" + "\n".join(lines) + "\n")
    host = read_matrix_market(p)
    dev = read_matrix_market(p, out="device")
    assert csr_bits_equal(to_host(dev), host)
    got = engine.multiply(dev, dev)
    want = port.serial_spgemm(host, host)
    assert csr_bits_equal(got, want), explain_diff(got, want)
