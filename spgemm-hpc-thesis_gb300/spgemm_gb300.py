"""Python binding of the GB300 SpGEMM engine (libspgemm_gb300.so, C ABI in
include/spgemm_gb300.h) and of the synthetic-input generators (libspg_synth.so).

The engine is the only compute path: there is no CPU fallback.  Loading the
library fails loudly when it has not been built (``python build.py`` in this
directory, or ``__graft_entry__.build()``).

Host matrices are ``Csr`` (numpy int64 row offsets, int32 columns, float64
values, the reference's CsrMatrix layout).  Device matrices are ``DeviceCsr``
(torch CUDA tensors of the same dtypes); torch is used only to own device
memory.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libspgemm_gb300.so"
SYNTH_PATH = HERE / "libspg_synth.so"

SPG_HOST, SPG_DEVICE = 0, 1
STATUS_NAMES = {0: "SPG_OK", 1: "SPG_INVALID_ARGUMENT", 2: "SPG_OVERFLOW", 3: "SPG_OUT_OF_RANGE_COLUMN",
                4: "SPG_OUT_OF_MEMORY", 5: "SPG_BUDGET_EXCEEDED", 6: "SPG_DEVICE_TIMEOUT", 7: "SPG_CUDA_ERROR",
                8: "SPG_NOT_READY", 9: "SPG_CANCELLED", 10: "SPG_FORMAT_ERROR"}
BIN_NAMES = ["empty", "w<=32", "w<=64", "w<=96", "w<=128", "w<=192", "w<=256", "w<=384", "w<=512", "b<=768",
             "b<=1K", "b<=1.5K", "b<=2K", "b<=3K", "b<=4K", "b<=6K", "b<=8K", "b<=12K", "b<=16K", "heavy"]


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

    @staticmethod
    def from_arrays(rows, cols, row_ptr, col, val) -> "Csr":
        return Csr(int(rows), int(cols), np.ascontiguousarray(row_ptr, dtype=np.int64),
                   np.ascontiguousarray(col, dtype=np.int32), np.ascontiguousarray(val, dtype=np.float64))

    def to_device(self, device: int = 0) -> "DeviceCsr":
        import torch
        dev = torch.device("cuda", device)
        return DeviceCsr(self.rows, self.cols, torch.from_numpy(np.ascontiguousarray(self.row_ptr)).to(dev),
                         torch.from_numpy(np.ascontiguousarray(self.col)).to(dev),
                         torch.from_numpy(np.ascontiguousarray(self.val)).to(dev))

    def scaled(self, factor: float) -> "Csr":
        return Csr(self.rows, self.cols, self.row_ptr.copy(), self.col.copy(), self.val * factor)


@dataclass
class DeviceCsr:
    rows: int
    cols: int
    row_ptr: object  # torch.int64 CUDA tensor
    col: object      # torch.int32
    val: object      # torch.float64

    @property
    def nnz(self) -> int:
        return int(self.col.numel())


class SpgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.name = STATUS_NAMES.get(status, str(status))


class _View(C.Structure):
    _fields_ = [("rows", C.c_int32), ("cols", C.c_int32), ("nnz", C.c_int64), ("row_ptr", C.c_void_p),
                ("col", C.c_void_p), ("val", C.c_void_p), ("location", C.c_int32)]


class _Result(C.Structure):
    _fields_ = [("rows", C.c_int32), ("cols", C.c_int32), ("nnz", C.c_int64), ("row_ptr", C.c_void_p),
                ("col", C.c_void_p), ("val", C.c_void_p), ("location", C.c_int32), ("reserved", C.c_int32),
                ("products", C.c_int64)]


class _Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("mode", C.c_int32), ("hbm_budget_bytes", C.c_uint64),
                ("bin_streams", C.c_int32), ("reserved", C.c_int32)]


MODES = {"auto": 0, "exact": 1, "upper_bound": 2}


class Timings(C.Structure):
    _fields_ = [("ms_rowwork", C.c_float), ("ms_symbolic", C.c_float), ("ms_scan", C.c_float),
                ("ms_numeric", C.c_float), ("ms_compact", C.c_float), ("ms_total", C.c_float),
                ("products", C.c_int64), ("nnz", C.c_int64), ("rows", C.c_int64), ("bin_rows", C.c_int64 * 20),
                ("launches", C.c_int64), ("ms_numeric_bin", C.c_float * 20)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("bin_rows", "ms_numeric_bin")}
        d["bin_rows"] = {BIN_NAMES[i]: int(self.bin_rows[i]) for i in range(len(BIN_NAMES))}
        d["ms_numeric_bin"] = {BIN_NAMES[i]: float(self.ms_numeric_bin[i]) for i in range(len(BIN_NAMES))}
        return d


class FullReport(C.Structure):
    _fields_ = [("passed", C.c_int32), ("environment_ok", C.c_int32), ("matrices_ok", C.c_int32),
                ("partial_passed", C.c_int32), ("rejected", C.c_int64), ("row_nnz_mismatches", C.c_int64),
                ("support_mismatches", C.c_int64), ("reference_nnz", C.c_int64),
                ("checked_coordinates", C.c_int64), ("max_abs_error", C.c_double),
                ("max_error_ratio", C.c_double), ("max_rel_error", C.c_double), ("median_rel_error", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class TuneReport(C.Structure):
    _fields_ = [("ms_bin", (C.c_float * 20) * 2), ("bin_rows", C.c_int64 * 20), ("products", C.c_int64),
                ("variant", C.c_uint8 * 20)]

    def as_dict(self) -> dict:
        bins = {}
        for i, name in enumerate(BIN_NAMES):
            if self.bin_rows[i]:
                bins[name] = {"ms_default": round(self.ms_bin[0][i], 4), "ms_alt": round(self.ms_bin[1][i], 4),
                              "variant": int(self.variant[i])}
        return {"products": int(self.products), "bins": bins, "variants": list(self.variant)}


class _SynthCsr(C.Structure):
    _fields_ = [("rows", C.c_int32), ("cols", C.c_int32), ("nnz", C.c_int64),
                ("row_ptr", C.POINTER(C.c_int64)), ("col", C.POINTER(C.c_int32)), ("val", C.POINTER(C.c_double))]


_lib = None


def library() -> C.CDLL:
    """The engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA engine first (python build.py)")
        lib = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW)
        lib.spg_last_error.restype = C.c_char_p
        lib.spg_last_error.argtypes = [C.c_void_p]
        lib.spg_status_string.restype = C.c_char_p
        lib.spg_stream.restype = C.c_void_p
        lib.spg_stream.argtypes = [C.c_void_p]
        lib.spg_host_alloc.restype = C.c_void_p
        lib.spg_host_alloc.argtypes = [C.c_size_t]
        lib.spg_host_free.argtypes = [C.c_void_p]
        lib.spg_destroy.argtypes = [C.c_void_p]
        lib.spg_server_destroy.argtypes = [C.c_void_p]
        lib.spg_server_destroy.restype = None
        lib.spg_csr_release.argtypes = [C.c_void_p]
        lib.spg_csr_release.restype = None
        lib.spg_plan_destroy.argtypes = [C.c_void_p]
        lib.spg_plan_destroy.restype = None
        lib.spg_plan_last_ms.argtypes = [C.c_void_p]
        lib.spg_plan_last_ms.restype = C.c_float
        for name in ("spg_multiply", "spg_multiply_batch", "spg_accum_begin", "spg_accum_add", "spg_accum_finish",
                     "spg_result_download", "spg_result_free", "spg_scalar_multiplication_count",
                     "spg_scalar_multiplication_count_batch", "spg_last_timings", "spg_create", "spg_multiply_to_host",
                     "spg_config_default", "spg_server_create", "spg_submit", "spg_poll", "spg_cancel",
                     "spg_server_result_free", "spg_plan_create", "spg_plan_execute", "spg_plan_result", "spg_tune",
                     "spg_get_bin_variants", "spg_set_bin_variants", "spg_validate_full", "spg_transpose",
                     "spg_read_matrix_market", "spg_partition_rows"):
            getattr(lib, name).restype = C.c_int
        _lib = lib
    return _lib


def _host_view(m: Csr, keep: list) -> _View:
    rp = np.ascontiguousarray(m.row_ptr, dtype=np.int64)
    ci = np.ascontiguousarray(m.col, dtype=np.int32)
    va = np.ascontiguousarray(m.val, dtype=np.float64)
    keep += [rp, ci, va]
    return _View(int(m.rows), int(m.cols), int(rp[-1]) if len(rp) else 0, rp.ctypes.data,
                 ci.ctypes.data if ci.size else None, va.ctypes.data if va.size else None, SPG_HOST)


def _dev_view(m: DeviceCsr) -> _View:
    import torch
    assert m.row_ptr.dtype == torch.int64 and m.col.dtype == torch.int32 and m.val.dtype == torch.float64
    return _View(int(m.rows), int(m.cols), int(m.col.numel()), m.row_ptr.data_ptr(),
                 m.col.data_ptr() if m.col.numel() else None, m.val.data_ptr() if m.val.numel() else None,
                 SPG_DEVICE)


def _view(m, keep: list) -> _View:
    return _dev_view(m) if isinstance(m, DeviceCsr) else _host_view(m, keep)


class DeviceResult:
    """A result held in device memory owned by the engine."""

    def __init__(self, engine: "Engine", res: _Result):
        self._engine = engine
        self._res = res
        self.rows, self.cols, self.nnz, self.products = res.rows, res.cols, res.nnz, res.products

    @property
    def pointers(self) -> tuple[int, int, int]:
        return self._res.row_ptr, self._res.col, self._res.val

    def download(self) -> Csr:
        rp = np.empty(self.rows + 1, dtype=np.int64)
        ci = np.empty(self.nnz, dtype=np.int32)
        va = np.empty(self.nnz, dtype=np.float64)
        self._engine._check(library().spg_result_download(
            self._engine.h, C.byref(self._res), rp.ctypes.data_as(C.c_void_p),
            ci.ctypes.data_as(C.c_void_p) if self.nnz else None, va.ctypes.data_as(C.c_void_p) if self.nnz else None))
        return Csr(self.rows, self.cols, rp, ci, va)

    def free(self):
        if self._res is not None and self._engine.h:
            library().spg_result_free(self._engine.h, C.byref(self._res))
        self._res = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _take_host(res: _Result, engine: "Engine") -> Csr:
    rows, nnz = res.rows, res.nnz
    rp = np.ctypeslib.as_array(C.cast(res.row_ptr, C.POINTER(C.c_int64)), shape=(rows + 1,)).copy()
    if nnz:
        ci = np.ctypeslib.as_array(C.cast(res.col, C.POINTER(C.c_int32)), shape=(nnz,)).copy()
        va = np.ctypeslib.as_array(C.cast(res.val, C.POINTER(C.c_double)), shape=(nnz,)).copy()
    else:
        ci, va = np.zeros(0, np.int32), np.zeros(0, np.float64)
    library().spg_result_free(engine.h, C.byref(res))
    return Csr(rows, res.cols, rp, ci, va)


class Engine:
    """One engine handle (one CUDA stream and its workspace) on one device."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, mode: str = "auto", bin_streams: int = 0):
        lib = library()
        cfg = _Config(device, MODES[mode], hbm_budget_bytes, bin_streams, 0)
        h = C.c_void_p()
        st = lib.spg_create(C.byref(cfg), C.byref(h))
        if st != 0:
            raise SpgError(st, "spg_create failed (no usable CUDA device?)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            library().spg_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != 0:
            raise SpgError(st, library().spg_last_error(self.h).decode())

    @property
    def stream(self) -> int:
        return library().spg_stream(self.h)

    def multiply(self, a, b, out: str = "host"):
        """C = A * B.  out="host" returns a Csr, out="device" a DeviceResult."""
        keep: list = []
        va, vb = _view(a, keep), _view(b, keep)
        res = _Result()
        loc = SPG_DEVICE if out == "device" else SPG_HOST
        self._check(library().spg_multiply(self.h, C.byref(va), C.byref(vb), C.c_int32(loc), C.byref(res)))
        return DeviceResult(self, res) if loc == SPG_DEVICE else _take_host(res, self)

    def multiply_to_host(self, a, b, row_ptr, col, val) -> int:
        """C = A * B into caller host arrays (numpy or pinned torch CPU tensors:
        row_ptr int64[A.rows+1], col int32[cap], val float64[cap]); returns
        nnz(C).  Device->host copies of finished row blocks overlap the rest."""
        keep: list = []
        va, vb = _view(a, keep), _view(b, keep)

        def ptr(x):
            return x.data_ptr() if hasattr(x, "data_ptr") else x.ctypes.data

        cap = min(len(col), len(val))
        nnz = C.c_int64()
        self._check(library().spg_multiply_to_host(self.h, C.byref(va), C.byref(vb), C.c_void_p(ptr(row_ptr)),
                                                   C.c_void_p(ptr(col)), C.c_void_p(ptr(val)), C.c_int64(cap),
                                                   C.byref(nnz)))
        return nnz.value

    def multiply_batch(self, pairs, out: str = "host") -> list:
        keep: list = []
        n = len(pairs)
        A = (_View * max(n, 1))(*[_view(a, keep) for a, _ in pairs])
        B = (_View * max(n, 1))(*[_view(b, keep) for _, b in pairs])
        R = (_Result * max(n, 1))()
        loc = SPG_DEVICE if out == "device" else SPG_HOST
        self._check(library().spg_multiply_batch(self.h, C.c_int32(n), A, B, C.c_int32(loc), R))
        return [DeviceResult(self, R[i]) if loc == SPG_DEVICE else _take_host(R[i], self) for i in range(n)]

    def accumulate(self, rows: int, cols: int, stages, out: str = "host"):
        """LocalAccumulator(rows, cols); addProduct(A, B) per stage; finish()."""
        lib = library()
        self._check(lib.spg_accum_begin(self.h, C.c_int32(rows), C.c_int32(cols)))
        for a, b in stages:
            keep: list = []
            va, vb = _view(a, keep), _view(b, keep)
            self._check(lib.spg_accum_add(self.h, C.byref(va), C.byref(vb)))
        res = _Result()
        loc = SPG_DEVICE if out == "device" else SPG_HOST
        self._check(lib.spg_accum_finish(self.h, C.c_int32(loc), C.byref(res)))
        self._check(lib.spg_accum_end(self.h))
        return DeviceResult(self, res) if loc == SPG_DEVICE else _take_host(res, self)

    def transpose(self, a, out: str = "host"):
        """spg_transpose: A^T with every row in A's row-major order."""
        keep: list = []
        va = _view(a, keep)
        res = _Result()
        loc = SPG_DEVICE if out == "device" else SPG_HOST
        self._check(library().spg_transpose(self.h, C.byref(va), C.c_int32(loc), C.byref(res)))
        return DeviceResult(self, res) if loc == SPG_DEVICE else _take_host(res, self)

    def validate_full(self, a, b, c) -> dict:
        """spg_validate_full: the reference's Full and Partial checks of C against A * B, on the GPU."""
        keep: list = []
        va, vb = _view(a, keep), _view(b, keep)
        if isinstance(c, DeviceResult):
            vc = _View(c.rows, c.cols, c.nnz, c._res.row_ptr, c._res.col, c._res.val, SPG_DEVICE)
        else:
            vc = _view(c, keep)
        rep = FullReport()
        self._check(library().spg_validate_full(self.h, C.byref(va), C.byref(vb), C.byref(vc), C.byref(rep)))
        return rep.as_dict()

    def tune(self, a, b, reps: int = 3) -> dict:
        """spg_tune: per-bin choice between the default and the alternative team shape."""
        keep: list = []
        va, vb = _view(a, keep), _view(b, keep)
        rep = TuneReport()
        self._check(library().spg_tune(self.h, C.byref(va), C.byref(vb), C.c_int32(reps), C.byref(rep)))
        return rep.as_dict()

    @property
    def bin_variants(self) -> list[int]:
        v = (C.c_uint8 * 20)()
        self._check(library().spg_get_bin_variants(self.h, v))
        return list(v)

    @bin_variants.setter
    def bin_variants(self, values) -> None:
        v = (C.c_uint8 * 20)(*values)
        self._check(library().spg_set_bin_variants(self.h, v))

    def plan(self, pairs) -> "Plan":
        return Plan(self, pairs)

    def scalar_multiplication_count_batch(self, pairs) -> list[int]:
        keep: list = []
        n = len(pairs)
        A = (_View * max(n, 1))(*[_view(a, keep) for a, _ in pairs])
        B = (_View * max(n, 1))(*[_view(b, keep) for _, b in pairs])
        P = (C.c_int64 * max(n, 1))()
        self._check(library().spg_scalar_multiplication_count_batch(self.h, C.c_int32(n), A, B, P))
        return [int(P[i]) for i in range(n)]

    def partition_rows(self, a, b, parts: int) -> np.ndarray:
        """spg_partition_rows: first_row[0..parts] cutting A's rows into blocks of
        about equal scalar products (device row work)."""
        keep: list = []
        va, vb = _view(a, keep), _view(b, keep)
        out = (C.c_int32 * (parts + 1))()
        self._check(library().spg_partition_rows(self.h, C.byref(va), C.byref(vb), C.c_int32(parts), out))
        return np.frombuffer(out, dtype=np.int32).copy()

    def scalar_multiplication_count(self, a, b) -> int:
        keep: list = []
        va, vb = _view(a, keep), _view(b, keep)
        n = C.c_int64()
        self._check(library().spg_scalar_multiplication_count(self.h, C.byref(va), C.byref(vb), C.byref(n)))
        return n.value

    def last_timings(self) -> dict:
        t = Timings()
        self._check(library().spg_last_timings(self.h, C.byref(t)))
        return t.as_dict()


class Plan:
    """spg_plan_*: the structure-dependent phases of n device-resident products
    once, the value-dependent ones as a CUDA graph replayed by execute()."""

    def __init__(self, engine: "Engine", pairs):
        self._engine = engine
        keep: list = []
        n = len(pairs)
        for a, b in pairs:
            if not isinstance(a, DeviceCsr) or not isinstance(b, DeviceCsr):
                raise TypeError("a plan needs DeviceCsr operands")
        A = (_View * n)(*[_view(a, keep) for a, _ in pairs])
        B = (_View * n)(*[_view(b, keep) for _, b in pairs])
        p = C.c_void_p()
        engine._check(library().spg_plan_create(engine.h, C.c_int32(n), A, B, C.byref(p)))
        self.p, self.n, self._pairs = p, n, pairs

    def execute(self) -> list[int]:
        nnz = (C.c_int64 * self.n)()
        self._engine._check(library().spg_plan_execute(self.p, nnz))
        return [int(x) for x in nnz]

    @property
    def last_ms(self) -> float:
        return float(library().spg_plan_last_ms(self.p))

    def result(self, i: int) -> Csr:
        """Host copy of product i of the last execution."""
        res = _Result()
        st = library().spg_plan_result(self.p, C.c_int32(i), C.byref(res))
        if st != 0:
            raise SpgError(st, "spg_plan_result failed (executed? index?)")
        rp = np.empty(res.rows + 1, dtype=np.int64)
        ci = np.empty(res.nnz, dtype=np.int32)
        va = np.empty(res.nnz, dtype=np.float64)
        self._engine._check(library().spg_result_download(
            self._engine.h, C.byref(res), rp.ctypes.data_as(C.c_void_p),
            ci.ctypes.data_as(C.c_void_p) if res.nnz else None, va.ctypes.data_as(C.c_void_p) if res.nnz else None))
        return Csr(res.rows, res.cols, rp, ci, va)

    def close(self):
        if getattr(self, "p", None):
            library().spg_plan_destroy(self.p)
            self.p = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _cudart() -> C.CDLL:
    """The CUDA runtime the engine library is linked against (already loaded
    with it): found by its soname, else by its path in this process's maps."""
    library()
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            return C.CDLL(name)
        except OSError:
            pass
    with open("/proc/self/maps") as f:
        for line in f:
            path = line.split()[-1]
            if "libcudart.so" in path:
                return C.CDLL(path)
    raise RuntimeError("the CUDA runtime library is not loaded")


def read_matrix_market(path, out: str = "host"):
    """spg_read_matrix_market: the reference's readMatrixMarket semantics
    (matrix_market.cpp:28-145).  out="host" returns a Csr; out="device" a
    DeviceCsr (torch tensors holding a copy of the library's device arrays)."""
    lib = library()
    res = _Result()
    err = C.create_string_buffer(256)
    loc = SPG_DEVICE if out == "device" else SPG_HOST
    st = lib.spg_read_matrix_market(str(path).encode(), C.c_int32(loc), C.byref(res), err, C.c_size_t(256))
    if st != 0:
        raise SpgError(st, err.value.decode(errors="replace"))
    try:
        if loc == SPG_HOST:
            rows, nnz = res.rows, res.nnz
            rp = np.ctypeslib.as_array(C.cast(res.row_ptr, C.POINTER(C.c_int64)), shape=(rows + 1,)).copy()
            ci = (np.ctypeslib.as_array(C.cast(res.col, C.POINTER(C.c_int32)), shape=(nnz,)).copy() if nnz
                  else np.zeros(0, np.int32))
            va = (np.ctypeslib.as_array(C.cast(res.val, C.POINTER(C.c_double)), shape=(nnz,)).copy() if nnz
                  else np.zeros(0, np.float64))
            return Csr(rows, res.cols, rp, ci, va)
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        rp = torch.empty(res.rows + 1, dtype=torch.int64, device=dev)
        ci = torch.empty(max(res.nnz, 1), dtype=torch.int32, device=dev)
        va = torch.empty(max(res.nnz, 1), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        cudart = _cudart()
        for dst, src, nb in ((rp, res.row_ptr, 8 * (res.rows + 1)), (ci, res.col, 4 * res.nnz), (va, res.val, 8 * res.nnz)):
            if nb and cudart.cudaMemcpy(C.c_void_p(dst.data_ptr()), C.c_void_p(src), C.c_size_t(nb), 3) != 0:
                raise SpgError(7, "device copy failed")
        return DeviceCsr(res.rows, res.cols, rp, ci[:res.nnz], va[:res.nnz])
    finally:
        lib.spg_csr_release(C.byref(res))


class _ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("lanes", C.c_int32), ("max_batch", C.c_int32), ("out_location", C.c_int32),
                ("mode", C.c_int32), ("reserved", C.c_int32), ("hbm_budget_bytes", C.c_uint64),
                ("max_batch_products", C.c_int64)]


class RequestInfo(C.Structure):
    _fields_ = [("queue_ms", C.c_double), ("service_ms", C.c_double), ("latency_ms", C.c_double),
                ("products", C.c_int64), ("footprint_bytes", C.c_int64), ("batch_requests", C.c_int32),
                ("lane", C.c_int32), ("batch_id", C.c_uint64), ("batch_launches", C.c_int64),
                ("message", C.c_char * 160)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "message"}
        d["message"] = self.message.decode(errors="replace")
        return d


class ServerResult:
    """A result delivered by a Server (device or host memory owned by the library)."""

    def __init__(self, server: "Server", res: _Result):
        self._server = server
        self._res = res
        self.rows, self.cols, self.nnz, self.products = res.rows, res.cols, res.nnz, res.products
        self.location = res.location

    def download(self) -> Csr:
        if self.location == SPG_HOST:
            rp = np.ctypeslib.as_array(C.cast(self._res.row_ptr, C.POINTER(C.c_int64)), shape=(self.rows + 1,)).copy()
            if self.nnz:
                ci = np.ctypeslib.as_array(C.cast(self._res.col, C.POINTER(C.c_int32)), shape=(self.nnz,)).copy()
                va = np.ctypeslib.as_array(C.cast(self._res.val, C.POINTER(C.c_double)), shape=(self.nnz,)).copy()
            else:
                ci, va = np.zeros(0, np.int32), np.zeros(0, np.float64)
            return Csr(self.rows, self.cols, rp, ci, va)
        eng = self._server._engine()
        rp = np.empty(self.rows + 1, dtype=np.int64)
        ci = np.empty(self.nnz, dtype=np.int32)
        va = np.empty(self.nnz, dtype=np.float64)
        eng._check(library().spg_result_download(
            eng.h, C.byref(self._res), rp.ctypes.data_as(C.c_void_p),
            ci.ctypes.data_as(C.c_void_p) if self.nnz else None, va.ctypes.data_as(C.c_void_p) if self.nnz else None))
        return Csr(self.rows, self.cols, rp, ci, va)

    def free(self):
        if self._res is not None and self._server.s:
            library().spg_server_result_free(self._server.s, C.byref(self._res))
        self._res = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """Serving loop (spg_server_*): submit products as they arrive, poll for
    results; batches of queued requests run together on `lanes` streams."""

    def __init__(self, device: int = 0, lanes: int = 2, max_batch: int = 256, out: str = "device",
                 mode: str = "auto", hbm_budget_bytes: int = 150 * 10**9, max_batch_products: int = 1 << 28):
        lib = library()
        cfg = _ServerConfig(device, lanes, max_batch, SPG_DEVICE if out == "device" else SPG_HOST, MODES[mode], 0,
                            int(hbm_budget_bytes), int(max_batch_products))
        s = C.c_void_p()
        st = lib.spg_server_create(C.byref(cfg), C.byref(s))
        if st != 0:
            raise SpgError(st, "spg_server_create failed")
        self.s = s
        self.device = device
        self._keep: dict = {}
        self._eng = None

    def _engine(self) -> Engine:
        if self._eng is None:
            self._eng = Engine(self.device)
        return self._eng

    def submit(self, a, b) -> int:
        keep: list = []
        va, vb = _view(a, keep), _view(b, keep)
        t = C.c_uint64()
        st = library().spg_submit(self.s, C.byref(va), C.byref(vb), C.byref(t))
        if st != 0:
            raise SpgError(st, "spg_submit failed")
        self._keep[t.value] = (keep, a, b)
        return t.value

    def poll(self, ticket: int, wait_ms: int = -1):
        """(status name, ServerResult or None, info dict); "SPG_NOT_READY" while it runs."""
        res, info = _Result(), RequestInfo()
        st = library().spg_poll(self.s, C.c_uint64(ticket), C.c_int32(wait_ms), C.byref(res), C.byref(info))
        if st == 8:
            return "SPG_NOT_READY", None, None
        self._keep.pop(ticket, None)
        return STATUS_NAMES.get(st, str(st)), (ServerResult(self, res) if st == 0 else None), info.as_dict()

    def cancel(self, ticket: int) -> str:
        return STATUS_NAMES.get(library().spg_cancel(self.s, C.c_uint64(ticket)), "?")

    def close(self):
        if getattr(self, "s", None):
            library().spg_server_destroy(self.s)
            self.s = None
            self._keep.clear()
        if getattr(self, "_eng", None) is not None:
            self._eng.close()
            self._eng = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Synthetic inputs (libspg_synth.so)
_synth = None


def _synth_lib() -> C.CDLL:
    global _synth
    if _synth is None:
        if not SYNTH_PATH.exists():
            raise RuntimeError(f"{SYNTH_PATH} is missing: build it first (python build.py)")
        _synth = C.CDLL(str(SYNTH_PATH), mode=os.RTLD_NOW)
        _synth.spg_synth_powerlaw.argtypes = [C.c_int32, C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_double,
                                              C.c_uint64, C.c_void_p]
        _synth.spg_synth_uniform.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_void_p]
        _synth.spg_synth_laplacian3d.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_void_p]
        _synth.spg_synth_restriction.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]
    return _synth


def _synth_take(out: _SynthCsr) -> Csr:
    rows, nnz = out.rows, out.nnz
    rp = np.ctypeslib.as_array(out.row_ptr, shape=(rows + 1,)).copy()
    ci = np.ctypeslib.as_array(out.col, shape=(max(nnz, 1),))[:nnz].copy()
    va = np.ctypeslib.as_array(out.val, shape=(max(nnz, 1),))[:nnz].copy()
    _synth_lib().spg_synth_free(C.byref(out))
    return Csr(rows, out.cols, rp, ci, va)


def synth_uniform(rows: int, cols: int, min_len: int, max_len: int | None = None, seed: int = 1) -> Csr:
    out = _SynthCsr()
    rc = _synth_lib().spg_synth_uniform(rows, cols, min_len, min_len if max_len is None else max_len, seed,
                                        C.byref(out))
    if rc:
        raise ValueError("invalid uniform generator arguments")
    return _synth_take(out)


def synth_powerlaw(n: int, mean: float = 24.0, sigma: float = 1.2, max_len: int = 20000, band: int = 2048,
                   band_frac: float = 0.7, seed: int = 1) -> Csr:
    out = _SynthCsr()
    if _synth_lib().spg_synth_powerlaw(n, mean, sigma, max_len, band, band_frac, seed, C.byref(out)):
        raise ValueError("invalid power-law generator arguments")
    return _synth_take(out)


def synth_laplacian3d(nx: int, ny: int | None = None, nz: int | None = None) -> Csr:
    out = _SynthCsr()
    if _synth_lib().spg_synth_laplacian3d(nx, ny or nx, nz or nx, C.byref(out)):
        raise ValueError("invalid grid")
    return _synth_take(out)


def synth_restriction(nx: int, ny: int | None = None, nz: int | None = None, transpose: bool = False) -> Csr:
    out = _SynthCsr()
    if _synth_lib().spg_synth_restriction(nx, ny or nx, nz or nx, int(transpose), C.byref(out)):
        raise ValueError("invalid grid (sizes must be even)")
    return _synth_take(out)


def scalar_products_host(a: Csr, b: Csr) -> int:
    """P = sum over A entries of nnz(B row) (numpy; for workload bookkeeping)."""
    blen = np.diff(b.row_ptr)
    return int(blen[a.col].sum()) if a.nnz else 0


def algorithmic_bytes(a: Csr, b: Csr, products: int, c_nnz: int) -> int:
    """Bytes a single pass must move: read A, one B row-offset pair per A entry,
    one B entry (column + value) per product, write C."""
    m = a.rows
    return 8 * (m + 1) + 12 * a.nnz + 16 * a.nnz + 12 * products + 8 * (m + 1) + 12 * c_nnz
