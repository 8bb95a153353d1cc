"""ctypes binding of the CPU checkers (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module.  ``Port`` wraps ``liboracle.so`` (the C++ restatement of the
reference algorithms, oracle/spgemm_oracle.cpp); ``Reference`` wraps
``_ref/libspgemm_ref.so`` (the reference's own sources, present only where the
reference tree was available at build time).

Matrices are passed as any object with ``rows, cols, row_ptr (int64),
col (int32), val (float64)`` attributes; results come back as ``Csr``.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


@dataclass
class Csr:
    rows: int
    cols: int
    row_ptr: np.ndarray
    col: np.ndarray
    val: np.ndarray

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1]) if len(self.row_ptr) else 0


class _In(C.Structure):
    _fields_ = [("rows", C.c_int32), ("cols", C.c_int32), ("nnz", C.c_int64),
                ("row_ptr", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p)]


class _Out(C.Structure):
    _fields_ = [("rows", C.c_int32), ("cols", C.c_int32), ("nnz", C.c_int64),
                ("row_ptr", C.POINTER(C.c_int64)), ("col", C.POINTER(C.c_int32)),
                ("val", C.POINTER(C.c_double))]


class FullReport(C.Structure):
    _fields_ = [("passed", C.c_int32), ("environment_ok", C.c_int32), ("matrices_ok", C.c_int32),
                ("pad", C.c_int32), ("rejected", C.c_int64), ("row_nnz_mismatches", C.c_int64),
                ("support_mismatches", C.c_int64), ("reference_nnz", C.c_int64),
                ("checked_coordinates", C.c_int64), ("max_abs_error", C.c_double),
                ("max_error_ratio", C.c_double), ("max_rel_error", C.c_double),
                ("median_rel_error", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "pad"}


class _RefValidation(C.Structure):
    _fields_ = [("passed", C.c_int32), ("row_nnz_mismatches", C.c_int32), ("rejected", C.c_int64),
                ("max_abs_error", C.c_double), ("max_error_ratio", C.c_double)]


class OracleError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


def _arrays(m):
    rp = np.ascontiguousarray(m.row_ptr, dtype=np.int64)
    ci = np.ascontiguousarray(m.col, dtype=np.int32)
    va = np.ascontiguousarray(m.val, dtype=np.float64)
    return rp, ci, va


def _view(m, keep: list) -> _In:
    rp, ci, va = _arrays(m)
    keep += [rp, ci, va]
    return _In(int(m.rows), int(m.cols), int(rp[-1]) if len(rp) else 0, rp.ctypes.data,
               ci.ctypes.data if len(ci) else None, va.ctypes.data if len(va) else None)


def _take(out: _Out, free) -> Csr:
    rows, nnz = out.rows, out.nnz
    rp = np.ctypeslib.as_array(out.row_ptr, shape=(rows + 1,)).copy()
    ci = np.ctypeslib.as_array(out.col, shape=(max(nnz, 1),))[:nnz].copy()
    va = np.ctypeslib.as_array(out.val, shape=(max(nnz, 1),))[:nnz].copy()
    free(C.byref(out))
    return Csr(rows, out.cols, rp, ci, va)


class _Lib:
    prefix = ""

    def __init__(self, path: Path):
        self.lib = C.CDLL(str(path), mode=os.RTLD_NOW)
        self._last_error = getattr(self.lib, f"{self.prefix}last_error")
        self._last_error.restype = C.c_char_p

    def _check(self, rc: int):
        if rc != 0:
            raise OracleError(rc, self._last_error().decode())

    def _call_out(self, name: str, *args) -> Csr:
        out = _Out()
        self._check(getattr(self.lib, self.prefix + name)(*args, C.byref(out)))
        return _take(out, getattr(self.lib, self.prefix + "free"))


class Port(_Lib):
    """The C++ restatement of the reference algorithms (oracle/spgemm_oracle.cpp)."""
    prefix = "orc_"

    def __init__(self, path: Path | None = None):
        super().__init__(path or HERE / "liboracle.so")
        self.lib.orc_accum_create.restype = C.c_void_p
        self.lib.orc_accum_create.argtypes = [C.c_int32, C.c_int32]
        self.lib.orc_accum_destroy.argtypes = [C.c_void_p]
        self.lib.orc_accum_add.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        self.lib.orc_accum_finish.argtypes = [C.c_void_p, C.c_void_p]

    def max_threads(self) -> int:
        return int(self.lib.orc_max_threads())

    def serial_spgemm(self, a, b) -> Csr:
        k = []
        return self._call_out("serial_spgemm", C.byref(_view(a, k)), C.byref(_view(b, k)))

    def serial_rows(self, a, b, rows) -> Csr:
        k = []
        r = np.ascontiguousarray(rows, dtype=np.int32)
        return self._call_out("serial_rows", C.byref(_view(a, k)), C.byref(_view(b, k)),
                              r.ctypes.data_as(C.c_void_p), C.c_int32(len(r)))

    def spgemm_omp(self, a, b, threads: int = 0, chunk: int = 64) -> Csr:
        k = []
        return self._call_out("spgemm_omp", C.byref(_view(a, k)), C.byref(_view(b, k)),
                              C.c_int(threads), C.c_int(chunk))

    def spgemm_omp_rows(self, a, b, first: int, count: int, threads: int = 0, chunk: int = 64) -> int:
        k = []
        nnz = C.c_int64()
        self._check(self.lib.orc_spgemm_omp_rows(C.byref(_view(a, k)), C.byref(_view(b, k)),
                                                 C.c_int32(first), C.c_int32(count), C.c_int(threads),
                                                 C.c_int(chunk), C.byref(nnz)))
        return nnz.value

    def scalar_multiplication_count(self, a, b) -> int:
        k = []
        n = C.c_int64()
        self._check(self.lib.orc_scalar_multiplication_count(C.byref(_view(a, k)), C.byref(_view(b, k)),
                                                             C.byref(n)))
        return n.value

    def partial_reference(self, a, b) -> tuple[np.ndarray, bool]:
        k = []
        counts = np.zeros(int(a.rows), dtype=np.int64)
        fin = C.c_int32()
        self._check(self.lib.orc_partial_reference(C.byref(_view(a, k)), C.byref(_view(b, k)),
                                                   counts.ctypes.data_as(C.c_void_p), C.byref(fin)))
        return counts, bool(fin.value)

    def compare_partial(self, counts: np.ndarray, finite: bool, rows: int, cols: int, c) -> tuple[bool, int]:
        k = []
        counts = np.ascontiguousarray(counts, dtype=np.int64)
        ok, mism = C.c_int32(), C.c_int64()
        self._check(self.lib.orc_compare_partial(counts.ctypes.data_as(C.c_void_p), C.c_int32(int(finite)),
                                                 C.c_int32(rows), C.c_int32(cols), C.byref(_view(c, k)),
                                                 C.byref(ok), C.byref(mism)))
        return bool(ok.value), mism.value

    def validate_partial(self, a, b, c) -> tuple[bool, int]:
        counts, fin = self.partial_reference(a, b)
        return self.compare_partial(counts, fin, int(a.rows), int(b.cols), c)

    def validate_full(self, a, b, c, rows=None) -> dict:
        k = []
        rep = FullReport()
        if rows is None:
            rp, n = None, 0
        else:
            r = np.ascontiguousarray(rows, dtype=np.int32)
            k.append(r)
            rp, n = r.ctypes.data_as(C.c_void_p), len(r)
        self._check(self.lib.orc_validate_full(C.byref(_view(a, k)), C.byref(_view(b, k)),
                                               C.byref(_view(c, k)), rp, C.c_int32(n), C.byref(rep)))
        return rep.as_dict()

    def read_mtx(self, path) -> Csr:
        return self._call_out("read_mtx", str(path).encode())

    def accumulate(self, rows: int, cols: int, stages) -> Csr:
        """LocalAccumulator(rows, cols); addProduct for each (A, B); finish()."""
        h = self.lib.orc_accum_create(rows, cols)
        try:
            for a, b in stages:
                k = []
                self._check(self.lib.orc_accum_add(h, C.byref(_view(a, k)), C.byref(_view(b, k))))
            out = _Out()
            self._check(self.lib.orc_accum_finish(h, C.byref(out)))
            return _take(out, self.lib.orc_free)
        finally:
            self.lib.orc_accum_destroy(h)


class Reference(_Lib):
    """The reference's own sources (oracle/_ref), built by oracle/build.py."""
    prefix = "ref_"

    @staticmethod
    def available() -> bool:
        return (HERE / "_ref" / "libspgemm_ref.so").exists()

    def __init__(self, path: Path | None = None):
        super().__init__(path or HERE / "_ref" / "libspgemm_ref.so")
        self.lib.ref_accum_create.restype = C.c_void_p
        self.lib.ref_accum_create.argtypes = [C.c_int32, C.c_int32]
        self.lib.ref_accum_destroy.argtypes = [C.c_void_p]
        self.lib.ref_accum_add.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        self.lib.ref_accum_finish.argtypes = [C.c_void_p, C.c_void_p]

    def serial_spgemm(self, a, b) -> Csr:
        k = []
        return self._call_out("serial_spgemm", C.byref(_view(a, k)), C.byref(_view(b, k)))

    def spgemm(self, a, b, threads: int = 0, chunk: int = 64) -> Csr:
        k = []
        return self._call_out("spgemm", C.byref(_view(a, k)), C.byref(_view(b, k)), C.c_int(threads),
                              C.c_int(chunk))

    def spgemm_timed(self, a, b, threads: int = 0, chunk: int = 64, repeats: int = 1):
        k = []
        secs = np.zeros(repeats, dtype=np.float64)
        nnz = C.c_int64()
        self._check(self.lib.ref_spgemm_timed(C.byref(_view(a, k)), C.byref(_view(b, k)), C.c_int(threads),
                                              C.c_int(chunk), C.c_int(repeats),
                                              secs.ctypes.data_as(C.c_void_p), C.byref(nnz)))
        return secs, nnz.value

    def scalar_multiplication_count(self, a, b) -> int:
        k = []
        n = C.c_int64()
        self._check(self.lib.ref_scalar_multiplication_count(C.byref(_view(a, k)), C.byref(_view(b, k)),
                                                             C.byref(n)))
        return n.value

    def validate(self, a, b, c, full: bool) -> dict:
        k = []
        v = _RefValidation()
        self._check(self.lib.ref_validate(C.byref(_view(a, k)), C.byref(_view(b, k)), C.byref(_view(c, k)),
                                          C.c_int(int(full)), C.byref(v)))
        return {"passed": bool(v.passed), "row_nnz_mismatches": v.row_nnz_mismatches,
                "rejected": v.rejected, "max_abs_error": v.max_abs_error,
                "max_error_ratio": v.max_error_ratio}

    def read_mtx(self, path) -> Csr:
        return self._call_out("read_mtx", str(path).encode())

    def accumulate(self, rows: int, cols: int, stages) -> Csr:
        h = self.lib.ref_accum_create(rows, cols)
        try:
            for a, b in stages:
                k = []
                self._check(self.lib.ref_accum_add(h, C.byref(_view(a, k)), C.byref(_view(b, k))))
            out = _Out()
            self._check(self.lib.ref_accum_finish(h, C.byref(out)))
            return _take(out, self.lib.ref_free)
        finally:
            self.lib.ref_accum_destroy(h)


def csr_equal_bits(x, y) -> bool:
    """Bitwise equality of two CSR matrices (values compared as raw 64-bit words)."""
    return (int(x.rows) == int(y.rows) and int(x.cols) == int(y.cols)
            and np.array_equal(np.asarray(x.row_ptr), np.asarray(y.row_ptr))
            and np.array_equal(np.asarray(x.col), np.asarray(y.col))
            and np.array_equal(np.asarray(x.val, dtype=np.float64).view(np.uint64),
                               np.asarray(y.val, dtype=np.float64).view(np.uint64)))
