"""The allocation-free multiply (spg_multiply_noalloc) through the C ABI.

This entry point serves callers that cannot allocate device memory when they
multiply (memory owned by another allocator or reserved at start-up, loops that
forbid allocator calls); its scratch is a fixed 32 MiB device array owned by
the library.  The test checks, on two calls in a row (the second finds the
first call's leftovers in the shared scratch), that its output equals the
regular spg_multiply's bit for bit, and that sizes beyond the scratch or the
output capacity are rejected.  It lives in its own file, collected last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import spgemm_gb300 as sg
from helpers import random_csr, row_sizes_for_bins

pytestmark = pytest.mark.gpu


def noalloc(lib, da, db, capacity: int):
    import torch
    dev = da.row_ptr.device
    rp = torch.zeros(da.rows + 1, dtype=torch.int64, device=dev)
    ci = torch.zeros(max(capacity, 1), dtype=torch.int32, device=dev)
    va = torch.zeros(max(capacity, 1), dtype=torch.float64, device=dev)
    nnz = C.c_int64(-1)
    err = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev).cuda_stream
    va_view, vb_view = sg._dev_view(da), sg._dev_view(db)
    st = lib.spg_multiply_noalloc(C.byref(va_view), C.byref(vb_view), C.c_void_p(stream), C.c_void_p(rp.data_ptr()),
                                  C.c_void_p(ci.data_ptr()), C.c_void_p(va.data_ptr()), C.c_int64(capacity),
                                  C.byref(nnz), err, C.c_size_t(256))
    if st != 0:
        return st, nnz.value, err.value.decode(), None
    n = nnz.value
    out = sg.Csr(da.rows, db.cols, rp.cpu().numpy(), ci[:n].cpu().numpy(), va[:n].cpu().numpy())
    return st, n, "", out


def same(x, y) -> bool:
    return (np.array_equal(x.row_ptr, y.row_ptr) and np.array_equal(x.col, y.col)
            and np.array_equal(x.val.view(np.uint64), y.val.view(np.uint64)))


def test_noalloc_matches_multiply_twice(port):
    lib = sg.library()
    lib.spg_multiply_noalloc.restype = C.c_int
    cases = [row_sizes_for_bins(3),
             (random_csr(500, 300, 40, 21, values="int"), random_csr(300, 200, 30, 22, values="int")),
             (random_csr(900, 700, 12, 23), random_csr(700, 800, 15, 24))]
    with sg.Engine(0) as eng:
        for a, b in cases:
            want = eng.multiply(a, b)
            assert same(want, port.serial_spgemm(a, b))  # both equal the serial reference product
            da, db = a.to_device(), b.to_device()
            for _ in range(2):  # the second call reuses the scratch left by the first
                st, n, msg, got = noalloc(lib, da, db, want.nnz)
                assert st == 0, msg
                assert n == want.nnz and same(got, want)


def test_noalloc_second_call_reserves_no_device_memory():
    # The first call on a device is the warm-up (it may load kernel code); a
    # second call on the same operands, into the same output arrays, must leave
    # the device's free memory unchanged.
    import torch
    lib = sg.library()
    lib.spg_multiply_noalloc.restype = C.c_int
    a, b = row_sizes_for_bins(5)
    da, db = a.to_device(), b.to_device()
    with sg.Engine(0) as eng:
        cap = eng.multiply(a, b).nnz
    rp = torch.zeros(da.rows + 1, dtype=torch.int64, device="cuda")
    ci = torch.zeros(cap, dtype=torch.int32, device="cuda")
    va = torch.zeros(cap, dtype=torch.float64, device="cuda")
    nnz = C.c_int64(-1)
    err = C.create_string_buffer(256)
    va_view, vb_view = sg._dev_view(da), sg._dev_view(db)
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        return lib.spg_multiply_noalloc(C.byref(va_view), C.byref(vb_view), C.c_void_p(stream),
                                        C.c_void_p(rp.data_ptr()), C.c_void_p(ci.data_ptr()),
                                        C.c_void_p(va.data_ptr()), C.c_int64(cap), C.byref(nnz), err,
                                        C.c_size_t(256))
    assert call() == 0, err.value
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    assert call() == 0, err.value
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert nnz.value == cap


def test_noalloc_rejects_beyond_limits():
    lib = sg.library()
    lib.spg_multiply_noalloc.restype = C.c_int
    a = random_csr(200, 150, 10, 31)
    b = random_csr(150, 170, 10, 32)
    with sg.Engine(0) as eng:
        want = eng.multiply(a, b)
    st, n, msg, _ = noalloc(lib, a.to_device(), b.to_device(), want.nnz - 1)
    assert sg.STATUS_NAMES[st] == "SPG_BUDGET_EXCEEDED" and n == want.nnz and "capacity" in msg
    big = random_csr(1_500_000, 10, 0, 33)  # row arrays alone exceed the fixed scratch
    small = random_csr(10, 10, 1, 34)
    st, _, msg, _ = noalloc(lib, big.to_device(), small.to_device(), 0)
    assert sg.STATUS_NAMES[st] == "SPG_BUDGET_EXCEEDED" and "32 MiB" in msg
    # still usable afterwards
    st, n, msg, got = noalloc(lib, a.to_device(), b.to_device(), want.nnz)
    assert st == 0 and same(got, want), msg
