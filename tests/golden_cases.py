"""Loader of tests/golden/golden.npz (outputs of the reference's own code,
generated by tests/golden/make_golden.py)."""
from __future__ import annotations

import json
from functools import lru_cache
from pathlib import Path

import numpy as np

from spgemm_gb300 import Csr

GOLDEN = Path(__file__).resolve().parent / "golden"


@lru_cache(maxsize=1)
def _data():
    return np.load(GOLDEN / "golden.npz"), json.loads((GOLDEN / "golden.json").read_text())


def matrix(key: str) -> Csr:
    z, _ = _data()
    rows, cols = (int(x) for x in z[key + ".shape"])
    r = z[key + ".r"]
    rp = np.zeros(rows + 1, dtype=np.int64)
    np.cumsum(np.bincount(r, minlength=rows), out=rp[1:])
    return Csr(rows, cols, rp, z[key + ".c"].astype(np.int32), z[key + ".v"].astype(np.float64))


def cases(kind: str) -> dict:
    _, idx = _data()
    return {k: v for k, v in sorted(idx.items()) if v["kind"] == kind}


def product_operands(name: str):
    meta = cases("product")[name]
    a = matrix(name + ".A")
    b = a if meta.get("b_is_a") else matrix(name + ".B")
    c = None if "error" in meta else matrix(name + ".C")
    return meta, a, b, c


def accumulate_operands(name: str):
    meta = cases("accumulate")[name]
    n = meta["stages"]
    if name == "accum_stages":
        b = matrix(name + ".B")
        stages = [(matrix(f"{name}.A{i}"), b) for i in range(n)]
    else:
        stages = [(matrix(f"{name}.A{i}"), matrix(f"{name}.B{i}")) for i in range(n)]
    return meta, stages, matrix(name + ".C")
