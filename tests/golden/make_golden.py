"""Generates tests/golden/golden.npz from the reference's own code.

Run in a checkout where the reference tree is available (REFERENCE_ROOT, else
a ``reference`` directory beside the repository): it builds oracle/_ref (the reference's sources,
compiled unchanged with a single-rank MPI stand-in), reads the reference's
Matrix Market fixtures with the reference's reader, and records for every case
the inputs and the outputs of the reference's serialSpgemm, spgemm() (the
baseline local multiply, 4 OpenMP threads), scalarMultiplicationCount,
trident::LocalAccumulator and validateProduct.  The GPU tests and the oracle
tests check themselves against this file; nothing reads the reference tree at
test time.

Inputs restated from the reference's tests (file:line of the reference):
  serial_known        tests/spgemm_serial_smoke.cpp:65-67 (expected {16, 15})
  serial_dense_<s>    tests/spgemm_serial_smoke.cpp:10-21, 33-36 (100 seeded cases)
  cancellation        tests/spgemm_validation_smoke.cpp:153-155
  order_keep/cancel   tests/partial_reference_test.cpp:151-157
  reorder_tiny        tests/spgemm_full_streaming.cpp:58-62
  trident_<shape>     tests/trident_correctness.cpp:58-76, 207-213
  accum_stages        tests/trident_accumulator_memory.cpp:40-57
  mtx_*               tests/data/*.mtx, matrices/*.mtx, tests/data/hv15r_roundoff/*
"""
from __future__ import annotations

import json
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import build as obuild  # noqa: E402
from oracle.oracle import Csr, OracleError, Reference  # noqa: E402


def csr(rows, cols, rp, ci, va) -> Csr:
    return Csr(rows, cols, np.asarray(rp, np.int64), np.asarray(ci, np.int32), np.asarray(va, np.float64))


def serial_smoke_input(rows, cols, salt) -> Csr:
    rp, ci, va = [0], [], []
    for row in range(rows):
        if cols and (row + salt) % 4:
            for entry in range(2 * cols + 1):
                ci.append((entry * 7 + row + salt) % cols)
                va.append(float((entry * 3 + row + salt) % 7 - 3))
        rp.append(len(va))
    return csr(rows, cols, rp, ci, va)


def trident_sparse_input(rows, cols, salt) -> Csr:
    rp, ci, va = [0], [], []
    for i in range(rows):
        for j in range(cols):
            if (i + salt) % 5 != 0 and (i * 13 + j * 7 + salt) % 4 != 0:
                v = (i * 3 + j * 11 + salt) % 9 - 4
                if v != 0:
                    ci.append(j)
                    va.append(float(v))
        rp.append(len(va))
    return csr(rows, cols, rp, ci, va)


def random_input(rows, cols, lens, seed, values="uniform") -> Csr:
    rng = np.random.default_rng(seed)
    lens = np.asarray(lens, np.int64)
    rp = np.concatenate([[0], np.cumsum(lens)])
    n = int(rp[-1])
    ci = rng.integers(0, max(cols, 1), size=n)
    va = rng.uniform(-1, 1, size=n) if values == "uniform" else rng.integers(-4, 5, size=n) * 0.125
    va[rng.random(n) < 0.05] = 0.0
    return csr(rows, cols, rp, ci, va)


class Store:
    def __init__(self):
        self.arrays: dict[str, np.ndarray] = {}
        self.index: dict[str, dict] = {}

    def put_matrix(self, key: str, m: Csr):
        # stored as (row of every entry, column, value) + shape: compact for tall, nearly empty matrices
        lens = np.diff(m.row_ptr)
        self.arrays[key + ".r"] = np.repeat(np.arange(m.rows, dtype=np.int32), lens)
        self.arrays[key + ".c"] = np.asarray(m.col, np.int32)
        self.arrays[key + ".v"] = np.asarray(m.val, np.float64)
        self.arrays[key + ".shape"] = np.array([m.rows, m.cols], np.int64)

    def case(self, name: str, **meta):
        self.index[name] = meta


def main():
    obuild.build_oracle()
    if obuild.build_ref() is None:
        raise SystemExit("reference tree not found (set REFERENCE_ROOT)")
    ref = Reference()
    root = obuild.reference_root()
    st = Store()

    def product_case(name, a, b, **extra):
        st.put_matrix(name + ".A", a)
        meta = {"kind": "product", **extra}
        if b is a:
            meta["b_is_a"] = True
        else:
            st.put_matrix(name + ".B", b)
        try:
            c = ref.serial_spgemm(a, b)
        except OracleError as e:
            meta["error"] = e.code
            st.case(name, **meta)
            return
        st.put_matrix(name + ".C", c)
        c_omp = ref.spgemm(a, b, threads=4)
        meta["baseline_equals_serial"] = bool(
            np.array_equal(c.row_ptr, c_omp.row_ptr) and np.array_equal(c.col, c_omp.col)
            and np.array_equal(c.val.view(np.uint64), c_omp.val.view(np.uint64)))
        meta["products"] = ref.scalar_multiplication_count(a, b)
        part = ref.validate(a, b, c, full=False)
        full = ref.validate(a, b, c, full=True)
        meta["partial_passed"] = part["passed"]
        meta["full_passed"] = full["passed"]
        meta["full_max_error_ratio"] = full["max_error_ratio"]
        st.case(name, **meta)

    product_case("serial_known", csr(2, 3, [0, 2, 3], [0, 2, 1], [1, 2, 3]),
                 csr(3, 2, [0, 1, 2, 3], [1, 0, 1], [4, 5, 6]))
    for seed in range(100):
        a = serial_smoke_input(seed % 8, (seed * 3) % 7, seed)
        b = serial_smoke_input(a.cols, (seed * 5) % 9, seed + 1)
        product_case(f"serial_dense_{seed}", a, b)
    product_case("cancellation", csr(3, 2, [0, 2, 2, 3], [0, 1, 1], [1, 1, 2]),
                 csr(2, 3, [0, 2, 4], [0, 1, 0, 2], [1, 2, -1, 3]))
    one = csr(1, 1, [0, 1], [0], [1.0])
    product_case("order_keep", one, csr(1, 1, [0, 3], [0, 0, 0], [1e16, -1e16, 1.0]))
    product_case("order_cancel", one, csr(1, 1, [0, 3], [0, 0, 0], [1e16, 1.0, -1e16]))
    tiny = math.ldexp(1.0, -55)
    product_case("reorder_tiny", csr(1, 3, [0, 3], [0, 1, 2], [1, 1, 1]),
                 csr(3, 1, [0, 1, 2, 3], [0, 0, 0], [1, tiny, -1]))
    for value, tag in ((1e200, "overflow"), (1e-200, "underflow"), (1.0, "unit")):
        m = csr(1, 1, [0, 1], [0], [value])
        product_case(f"square_{tag}", m, m)
    for shape in ((7, 9, 5), (1, 1, 1), (0, 3, 2), (3, 0, 4), (3, 4, 0), (19, 11, 13), (61, 67, 59)):
        m, k, n = shape
        product_case("trident_{}x{}x{}".format(*shape), trident_sparse_input(m, k, 1), trident_sparse_input(k, n, 2))
    product_case("trident_cancel", csr(2, 2, [0, 2, 4], [0, 1, 0, 1], [1, 1, 1, -1]),
                 csr(2, 2, [0, 2, 4], [0, 1, 0, 1], [1, -1, -1, 1]))
    product_case("trident_emptyA", csr(3, 4, [0, 0, 0, 0], [], []), trident_sparse_input(4, 2, 3))
    product_case("out_of_range_column", csr(1, 2, [0, 1], [5], [1.0]), csr(2, 2, [0, 1, 2], [0, 1], [1.0, 1.0]))
    for i, (m, k, n, la, lb, vals) in enumerate([(300, 200, 250, 14, 11, "uniform"), (120, 40, 60, 30, 20, "dyadic"),
                                                   (6, 1500, 3000, 300, 20, "uniform"),
                                                   (192, 2048, 2048, 16, 16, "uniform")]):
        a = random_input(m, k, np.full(m, la), 100 + i, vals)
        b = random_input(k, n, np.full(k, lb), 200 + i, vals)
        product_case(f"random_{i}", a, b)

    # LocalAccumulator stages (trident_accumulator_memory.cpp:40-57)
    a = csr(3, 2, [0, 3, 3, 4], [1, 0, 1, 0], [2.0, 1.0, -1.0, 3.0])
    b = csr(2, 4, [0, 3, 5], [3, 1, 3, 0, 1], [2.0, 4.0, -1.0, 5.0, -4.0])
    stages = [a, csr(3, 2, a.row_ptr, a.col, a.val * -1.0), csr(3, 2, a.row_ptr, a.col, a.val * -1.0 * -0.5)]
    acc = ref.accumulate(3, 4, [(s, b) for s in stages])
    for i, s in enumerate(stages):
        st.put_matrix(f"accum_stages.A{i}", s)
    st.put_matrix("accum_stages.B", b)
    st.put_matrix("accum_stages.C", acc)
    st.case("accum_stages", kind="accumulate", stages=3, rows=3, cols=4)
    rng = np.random.default_rng(7)
    rs = []
    for s in range(4):
        k = int(rng.integers(1, 30))
        rs.append((random_input(40, k, rng.integers(0, 10, size=40), 300 + s),
                   random_input(k, 35, rng.integers(0, 12, size=k), 400 + s, "dyadic")))
    acc = ref.accumulate(40, 35, rs)
    for i, (x, y) in enumerate(rs):
        st.put_matrix(f"accum_random.A{i}", x)
        st.put_matrix(f"accum_random.B{i}", y)
    st.put_matrix("accum_random.C", acc)
    st.case("accum_random", kind="accumulate", stages=4, rows=40, cols=35)

    # Matrix Market fixtures through the reference's reader
    data = root / "tests" / "data"
    mats = root / "matrices"
    reads = {}
    for p in sorted(data.glob("*.mtx")) + [mats / "cage8.mtx", mats / "cage8_restriction.mtx",
                                            mats / "permuted" / "cage8_permuted_s42.mtx"]:
        name = p.stem.replace("-", "_")
        try:
            m = ref.read_mtx(p)
            st.put_matrix(f"mtx_{name}", m)
            reads[name] = m
            st.case(f"mtx_{name}", kind="mtx", file=str(p.relative_to(root)))
        except OracleError as e:
            st.case(f"mtx_{name}", kind="mtx_error", file=str(p.relative_to(root)), error=e.code)
    for name in ("cancellation", "overflow", "overflow_product", "roundoff_stages", "tiny_symmetric", "empty",
                 "cage8", "cage8_permuted_s42"):
        product_case(f"mtxprod_{name}", reads[name], reads[name])
    product_case("mtxprod_rectangular", reads["rectangular_a"], reads["rectangular_b"])
    product_case("mtxprod_cage8_R", reads["cage8"], reads["cage8_restriction"])
    rt = reads["cage8_restriction"]
    hv = data / "hv15r_roundoff"
    for w in ("zero-cancellation-witness", "absolute-threshold-witness"):
        a = ref.read_mtx(hv / f"{w}-A.mtx")
        b = ref.read_mtx(hv / f"{w}-B.mtx")
        witness = json.loads((hv / f"{w}.json").read_text())
        product_case("hv15r_" + w.replace("-", "_"), a, b, witness_row=witness["row"], witness_col=witness["col"],
                     witness_serial=witness["serial"])
    del rt

    out = HERE / "golden.npz"
    np.savez_compressed(out, **st.arrays)
    (HERE / "golden.json").write_text(json.dumps(st.index, indent=1, sort_keys=True))
    print(f"{len(st.index)} cases, {out.stat().st_size / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
