"""Matrix Market reader (spg_read_matrix_market, host output, no GPU): the
reference's readMatrixMarket semantics (matrix_market.cpp:28-145) against the
oracle's restatement of it, on files covering every accepted form and every
rejected one."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import csr_bits_equal, explain_diff
from spgemm_gb300 import SpgError, read_matrix_market

GOOD = {
    "general": "%%MatrixMarket matrix coordinate real general\n% c\n\n3 4 5\n1 1 1.5\n3 4 -2\n1 2 3e2\n1 1 0.25\n2 3 4D-1\n",
    "symmetric": "%%MatrixMarket matrix coordinate real symmetric\n3 3 4\n1 1 2\n3 1 -1\n2 1 0.5\n3 3 7\n",
    "skew": "%%MatrixMarket matrix coordinate real skew-symmetric\n3 3 2\n2 1 1.25\n3 2 -4\n",
    "hermitian": "%%MatrixMarket Matrix Coordinate Real Hermitian\n2 2 2\n2 1 3\n1 1 1\n",
    "pattern": "%%MatrixMarket matrix coordinate pattern general\n2 3 3\n1 3\n2 1\n1 3\n",
    "integer": "%%MatrixMarket matrix coordinate integer general\n2 2 3\n1 2 7\n2 2 -3\n1 1 +4\n",
    "crlf_and_comments": "%%MatrixMarket matrix coordinate real general\r\n%x\r\n2 2 2\r\n%y\r\n1 1 1d0\r\n2 2 .5\r\n% trailing\r\n",
    "empty": "%%MatrixMarket matrix coordinate real general\n5 6 0\n",
    "fortran": "%%MatrixMarket matrix coordinate real general\n1 2 2\n1 2 1.0D+02\n1 1 -2.5d-3\n",
}

BAD = {
    "array": "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",
    "complex": "%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n",
    "banner": "%MatrixMarket matrix coordinate real general\n1 1 1\n1 1 1\n",
    "extra_header": "%%MatrixMarket matrix coordinate real general extra\n1 1 1\n1 1 1\n",
    "symmetry": "%%MatrixMarket matrix coordinate real diagonal\n1 1 1\n1 1 1\n",
    "no_size": "%%MatrixMarket matrix coordinate real general\n% only comments\n",
    "bad_size": "%%MatrixMarket matrix coordinate real general\n0 3 1\n1 1 1\n",
    "size_extra": "%%MatrixMarket matrix coordinate real general\n2 2 1 9\n1 1 1\n",
    "nonsquare_sym": "%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 1 1\n",
    "range": "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n",
    "zero_index": "%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1\n",
    "missing_value": "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1\n",
    "extra_token": "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1 1\n",
    "pattern_value": "%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 1 5\n",
    "inf": "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1e400\n",
    "skew_diag": "%%MatrixMarket matrix coordinate real skew-symmetric\n2 2 1\n1 1 1\n",
    "short": "%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1\n2 2 2\n",
    "long": "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1\n2 2 2\n",
    "float_index": "%%MatrixMarket matrix coordinate real general\n2 2 1\n1.5 1 1\n",
    "empty_file": "",
}


def write(tmp_path, name, text):
    p = tmp_path / f"{name}.mtx"
    p.write_bytes(text.encode())
    return p


@pytest.mark.parametrize("name", sorted(GOOD))
def test_accepted_files_match_the_oracle(tmp_path, port, name):
    p = write(tmp_path, name, GOOD[name])
    got = read_matrix_market(p)
    want = port.read_mtx(p)
    assert csr_bits_equal(got, want), explain_diff(got, want)
    from oracle.oracle import Reference
    if Reference.available():  # the reference's own reader, where it was built from its sources
        ref = Reference().read_mtx(p)
        assert csr_bits_equal(got, ref), explain_diff(got, ref)


@pytest.mark.parametrize("name", sorted(BAD))
def test_rejected_files_match_the_oracle(tmp_path, port, name):
    p = write(tmp_path, name, BAD[name])
    with pytest.raises(Exception):
        port.read_mtx(p)
    with pytest.raises(SpgError) as e:
        read_matrix_market(p)
    assert e.value.name == "SPG_FORMAT_ERROR"


def test_missing_file(tmp_path):
    with pytest.raises(SpgError) as e:
        read_matrix_market(tmp_path / "absent.mtx")
    assert e.value.name == "SPG_FORMAT_ERROR"


@pytest.mark.parametrize("symmetry", ["general", "symmetric", "skew-symmetric"])
def test_large_random_file_parsed_in_chunks(tmp_path, port, symmetry):
    # enough lines for every host thread's chunk, comments interleaved, duplicates kept in file order
    rng = np.random.default_rng(7)
    n, m = 3000, 40000
    r = rng.integers(1, n + 1, size=m)
    c = rng.integers(1, n + 1, size=m)
    if symmetry != "general":
        r, c = np.maximum(r, c), np.minimum(r, c)
        if symmetry == "skew-symmetric":
            keep = r != c
            r, c = r[keep], c[keep]
    v = rng.uniform(-1, 1, size=len(r))
    lines = [f"%%MatrixMarket matrix coordinate real {symmetry}", f"{n} {n} {len(r)}"]
    for i, (a, b, x) in enumerate(zip(r, c, v)):
        if i % 997 == 0:
            lines.append("% interleaved comment")
        lines.append(f"{a} {b} {float(x)!r}" if i % 3 else f"{a} {b} {float(x):.17e}".replace("e", "D"))
    p = write(tmp_path, "big", "\n".join(lines) + "\n")
    got = read_matrix_market(p)
    want = port.read_mtx(p)
    assert csr_bits_equal(got, want), explain_diff(got, want)
