// C++ drop-in layer over the C ABI (spgemm_gb300.h) for the reference's C++17
// host code.  Header only; link with -lspgemm_gb300.
//
// Every function is a template over the caller's CSR type, which must have the
// members of the reference's CsrMatrix (src/common/csr_matrix.hpp:43-49):
//   int rows, cols; std::vector<int64_t> rowPtr; std::vector<int> columnIndices;
//   std::vector<double> values.
// Statuses become the reference's exception types: std::invalid_argument for
// shapes and malformed input, std::overflow_error for counts, std::runtime_error
// for an A column outside B's rows (spgemm_common.cpp:141-143) and for a
// malformed Matrix Market file, std::bad_alloc for device memory.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "spgemm_gb300.h"

namespace spgemm_gb300 {

[[noreturn]] inline void throw_status(spg_status s, const std::string& msg) {
    switch (s) {
        case SPG_INVALID_ARGUMENT: throw std::invalid_argument(msg);
        case SPG_OVERFLOW: throw std::overflow_error(msg);
        case SPG_OUT_OF_MEMORY: throw std::bad_alloc();
        default: throw std::runtime_error(msg);
    }
}

template <class Csr>
spg_csr_view host_view(const Csr& m) {
    spg_csr_view v;
    v.rows = m.rows;
    v.cols = m.cols;
    v.nnz = static_cast<int64_t>(m.values.size());
    v.row_ptr = m.rowPtr.data();
    v.col = reinterpret_cast<const int32_t*>(m.columnIndices.data());
    v.val = m.values.data();
    v.location = SPG_HOST;
    return v;
}

// One engine handle (one CUDA stream and its device workspace).
class Engine {
public:
    explicit Engine(int device = 0, uint64_t hbm_budget_bytes = 0) {
        spg_config c;
        spg_config_default(&c);
        c.device = device;
        c.hbm_budget_bytes = hbm_budget_bytes;
        const spg_status s = spg_create(&c, &h_);
        if (s != SPG_OK) throw_status(s, "spg_create failed (no usable CUDA device)");
    }
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;
    ~Engine() { spg_destroy(h_); }

    spg_handle* handle() const { return h_; }

    void check(spg_status s) const {
        if (s != SPG_OK) throw_status(s, spg_last_error(h_));
    }

    // C = A * B, returned in the caller's CSR type.
    template <class Csr>
    Csr multiply(const Csr& a, const Csr& b) const {
        const spg_csr_view va = host_view(a), vb = host_view(b);
        spg_csr_result r;
        check(spg_multiply(h_, &va, &vb, SPG_DEVICE, &r));
        return download<Csr>(r);
    }

    template <class Csr>
    int64_t scalarMultiplicationCount(const Csr& a, const Csr& b) const {
        const spg_csr_view va = host_view(a), vb = host_view(b);
        int64_t n = 0;
        check(spg_scalar_multiplication_count(h_, &va, &vb, &n));
        return n;
    }

    // Moves a device result into a host CSR of the caller's type and frees it.
    template <class Csr>
    Csr download(spg_csr_result& r) const {
        Csr out;
        out.rows = r.rows;
        out.cols = r.cols;
        out.rowPtr.resize(static_cast<size_t>(r.rows) + 1);
        out.columnIndices.resize(static_cast<size_t>(r.nnz));
        out.values.resize(static_cast<size_t>(r.nnz));
        const spg_status s = spg_result_download(h_, &r, out.rowPtr.data(),
                                                 reinterpret_cast<int32_t*>(out.columnIndices.data()),
                                                 out.values.data());
        spg_result_free(h_, &r);
        check(s);
        return out;
    }

private:
    spg_handle* h_ = nullptr;
};

// The engine of the calling thread (handles are per thread; device 0 unless
// SPGEMM_GB300_DEVICE names another).
inline Engine& thread_engine() {
    thread_local Engine engine([] {
        const char* d = std::getenv("SPGEMM_GB300_DEVICE");
        return d ? std::atoi(d) : 0;
    }());
    return engine;
}

// Drop-in for serialSpgemm(A, B) (spgemm_common.hpp:80) and for the baseline
// spgemm(localA, RowBlock{0, B.rows}, B, RemoteSparseRows{}, comm)
// (spgemm_exchange.hpp:37-39) when every B row is local: the same CSR, bit for bit.
template <class Csr>
Csr spgemm(const Csr& a, const Csr& b) {
    return thread_engine().multiply(a, b);
}

// Drop-in for readMatrixMarket(path) (matrix_market.hpp; matrix_market.cpp:28-145):
// the same CsrMatrix, std::runtime_error for the same malformed files.
template <class Csr>
Csr readMatrixMarket(const std::string& path) {
    spg_csr_result r;
    char err[256] = {0};
    const spg_status s = spg_read_matrix_market(path.c_str(), SPG_HOST, &r, err, sizeof err);
    if (s != SPG_OK) throw_status(s, err);
    Csr out;
    out.rows = r.rows;
    out.cols = r.cols;
    out.rowPtr.assign(r.row_ptr, r.row_ptr + r.rows + 1);
    out.columnIndices.assign(r.col, r.col + r.nnz);
    out.values.assign(r.val, r.val + r.nnz);
    spg_csr_release(&r);
    return out;
}

// The reference's Full-mode verdict of validateProduct(A, B, C, ValidationMode::Full)
// (spgemm_common.cpp:720-851), computed on the GPU (the report also holds the
// Partial verdict of comparePartialReference, :541-572).
template <class Csr>
spg_full_report validateFull(const Csr& a, const Csr& b, const Csr& c, Engine& engine = thread_engine()) {
    const spg_csr_view va = host_view(a), vb = host_view(b), vc = host_view(c);
    spg_full_report rep;
    engine.check(spg_validate_full(engine.handle(), &va, &vb, &vc, &rep));
    return rep;
}

// A^T with every row in A's row-major order.
template <class Csr>
Csr transpose(const Csr& a, Engine& engine = thread_engine()) {
    const spg_csr_view va = host_view(a);
    spg_csr_result r;
    engine.check(spg_transpose(engine.handle(), &va, SPG_DEVICE, &r));
    return engine.template download<Csr>(r);
}

// Drop-in for trident::LocalAccumulator (matrix_blocks.hpp:23-32).  One
// accumulator per engine at a time (pass a separate Engine for a second one).
template <class Csr>
class LocalAccumulator {
public:
    LocalAccumulator(int rows, int cols, Engine& engine = thread_engine()) : e_(engine) {
        e_.check(spg_accum_begin(e_.handle(), rows, cols));
    }
    LocalAccumulator(const LocalAccumulator&) = delete;
    LocalAccumulator& operator=(const LocalAccumulator&) = delete;
    ~LocalAccumulator() { spg_accum_end(e_.handle()); }

    void addProduct(const Csr& a, const Csr& b) {
        const spg_csr_view va = host_view(a), vb = host_view(b);
        e_.check(spg_accum_add(e_.handle(), &va, &vb));
    }

    Csr finish() const {
        spg_csr_result r;
        e_.check(spg_accum_finish(e_.handle(), SPG_DEVICE, &r));
        return e_.template download<Csr>(r);
    }

private:
    Engine& e_;
};

}  // namespace spgemm_gb300
