"""The overflow contract (csr_matrix.hpp:13-41, pinned by the reference's
tests/csr_large_counts.cpp): a count that the engine cannot represent is
refused with SPG_OVERFLOW -- the C ABI's form of std::overflow_error -- before
anything is allocated for the result, and the handle stays usable.

The engine's representable limit is 2^30 scalar products in one output row
(every row is sorted in one pass whose positions are 32-bit).  The operands
that cross it are small: one row of A holding 2^15 entries that all point at
B's single row of 2^15 + 1 entries gives 2^30 + 2^15 products from under 1 MB
of input, the way the reference's test reaches its int64 boundaries without
allocating them."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import spgemm_gb300 as sg
from helpers import csr_bits_equal, random_csr

pytestmark = pytest.mark.gpu

LIMIT = 1 << 30


def over_limit_case():
    k, n = 1 << 15, (1 << 15) + 1
    a = sg.Csr.from_arrays(1, 1, [0, k], np.zeros(k, np.int32), np.full(k, 0.5))
    b = sg.Csr.from_arrays(1, n, [0, n], np.arange(n, dtype=np.int32), np.ones(n))
    assert k * n > LIMIT
    return a, b


@pytest.mark.parametrize("where", ["host", "device"])
def test_row_above_the_limit_is_refused(engine, where):
    a, b = over_limit_case()
    if where == "device":
        a, b = a.to_device(), b.to_device()
    assert engine.scalar_multiplication_count(a, b) == (1 << 15) * ((1 << 15) + 1)  # counting still works
    with pytest.raises(sg.SpgError) as e:
        engine.multiply(a, b)
    assert e.value.name == "SPG_OVERFLOW" and "2^30" in str(e.value)
    ok = engine.multiply(random_csr(30, 20, 5, 1), random_csr(20, 25, 4, 2))  # usable afterwards
    assert ok.rows == 30


def test_overflow_in_every_entry_point(engine):
    import torch
    a, b = over_limit_case()
    small_a, small_b = random_csr(30, 20, 5, 1), random_csr(20, 25, 4, 2)
    with pytest.raises(sg.SpgError) as e:
        engine.multiply_batch([(small_a, small_b), (a, b)])
    assert e.value.name == "SPG_OVERFLOW"
    rp, ci, va = np.empty(2, np.int64), np.empty(16, np.int32), np.empty(16, np.float64)
    with pytest.raises(sg.SpgError) as e:
        engine.multiply_to_host(a, b, rp, ci, va)
    assert e.value.name == "SPG_OVERFLOW"
    with pytest.raises(sg.SpgError) as e:
        engine.accumulate(1, b.cols, [(a, b)])
    assert e.value.name == "SPG_OVERFLOW"
    # the allocation-free entry point refuses it too, before touching its scratch
    lib = sg.library()
    lib.spg_multiply_noalloc.restype = C.c_int
    da, db = a.to_device(), b.to_device()
    out_rp = torch.zeros(2, dtype=torch.int64, device="cuda")
    out_c = torch.zeros(1, dtype=torch.int32, device="cuda")
    out_v = torch.zeros(1, dtype=torch.float64, device="cuda")
    nnz = C.c_int64(-1)
    err = C.create_string_buffer(256)
    va_, vb_ = sg._dev_view(da), sg._dev_view(db)
    st = lib.spg_multiply_noalloc(C.byref(va_), C.byref(vb_), C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                  C.c_void_p(out_rp.data_ptr()), C.c_void_p(out_c.data_ptr()),
                                  C.c_void_p(out_v.data_ptr()), C.c_int64(1), C.byref(nnz), err, C.c_size_t(256))
    assert sg.STATUS_NAMES[st] == "SPG_OVERFLOW", err.value
    got = engine.multiply(small_a, small_b)
    assert csr_bits_equal(got, engine.multiply(small_a, small_b))


def test_just_below_the_limit_counts_exactly(engine):
    # 2^15 entries of A on a B row of 2^15 - 1 entries: 2^30 - 2^15 products,
    # under the limit; only the count is taken (the product itself would need
    # 12 GB of scratch), and it is exact in int64.
    k, n = 1 << 15, (1 << 15) - 1
    a = sg.Csr.from_arrays(1, 1, [0, k], np.zeros(k, np.int32), np.full(k, 0.5))
    b = sg.Csr.from_arrays(1, n, [0, n], np.arange(n, dtype=np.int32), np.ones(n))
    assert engine.scalar_multiplication_count(a, b) == k * n < LIMIT
