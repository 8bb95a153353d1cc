// C entry points over the reference's own local-multiply sources, compiled in
// place from the read-only reference tree into oracle/_ref/libspgemm_ref.so by
// build_ref() in oracle/build.py.  TEST INFRASTRUCTURE ONLY: it pins the oracle
// restatement (oracle/spgemm_oracle.cpp) and generates the golden vectors.
//
// The reference's cached-oracle files (partial_reference.cpp,
// full_reference.cpp) need OpenSSL and a CMake-generated header; they are not
// compiled.  The six cache functions spgemm_common.cpp links against are
// defined below as refusals, so only the uncached validation paths run.
#include "spgemm_exchange.hpp"
#include "matrix_blocks.hpp"
#include "matrix_market.hpp"
#include "full_reference.hpp"

#include <cstring>
#include <iostream>
#include <sstream>
#include <stdexcept>

// ---- refusals for the cache layer (never reached without a cache directory)
std::string partialReferenceKey(const CsrMatrix&, const CsrMatrix&) {
    throw std::runtime_error("reference cache layer not built");
}
PartialReference readPartialReference(const std::filesystem::path&, const std::string&, int, int) {
    throw std::runtime_error("reference cache layer not built");
}
void printValidationDiagnostics(const ValidationDiagnostics&) {}
std::string fullReferenceKey(const CsrMatrix&, const CsrMatrix&) {
    throw std::runtime_error("reference cache layer not built");
}
struct FullReferenceReader::Impl {};
FullReferenceReader::FullReferenceReader(const std::filesystem::path&, const std::string&, int, int) {
    throw std::runtime_error("reference cache layer not built");
}
FullReferenceReader::~FullReferenceReader() = default;
void FullReferenceReader::readRow(FullReferenceRow&) {}
void FullReferenceReader::finish() {}
void prepareFullReferenceFile(const std::filesystem::path&, const std::string&, int, int,
                              const std::function<void(int, FullReferenceRow&)>&, ValidationDiagnostics&) {
    throw std::runtime_error("reference cache layer not built");
}

extern "C" {

typedef struct {
    int32_t rows, cols;
    int64_t nnz;
    const int64_t* row_ptr;
    const int32_t* col;
    const double* val;
} ref_csr;

typedef struct {
    int32_t rows, cols;
    int64_t nnz;
    int64_t* row_ptr;
    int32_t* col;
    double* val;
} ref_csr_out;

typedef struct {
    int32_t passed;
    int32_t row_nnz_mismatches;
    int64_t rejected;
    double max_abs_error;  // NaN when the reference reports none
    double max_error_ratio;
} ref_validation;

}  // extern "C"

namespace {
thread_local std::string last_error;

CsrMatrix to_matrix(const ref_csr* m) {
    CsrMatrix out;
    out.rows = m->rows;
    out.cols = m->cols;
    out.rowPtr.assign(m->row_ptr, m->row_ptr + m->rows + 1);
    out.columnIndices.assign(m->col, m->col + m->nnz);
    out.values.assign(m->val, m->val + m->nnz);
    return out;
}

void from_matrix(const CsrMatrix& m, ref_csr_out* out) {
    out->rows = m.rows;
    out->cols = m.cols;
    out->nnz = static_cast<int64_t>(m.values.size());
    out->row_ptr = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * m.rowPtr.size()));
    out->col = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (m.columnIndices.size() + 1)));
    out->val = static_cast<double*>(std::malloc(sizeof(double) * (m.values.size() + 1)));
    std::memcpy(out->row_ptr, m.rowPtr.data(), sizeof(int64_t) * m.rowPtr.size());
    if (!m.columnIndices.empty()) std::memcpy(out->col, m.columnIndices.data(), sizeof(int32_t) * m.columnIndices.size());
    if (!m.values.empty()) std::memcpy(out->val, m.values.data(), sizeof(double) * m.values.size());
}

template <typename F>
int guard(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::invalid_argument& e) {
        last_error = e.what();
        return 1;
    } catch (const std::overflow_error& e) {
        last_error = e.what();
        return 2;
    } catch (const std::exception& e) {
        last_error = e.what();
        return 3;
    }
}
}  // namespace

extern "C" {

const char* ref_last_error(void) { return last_error.c_str(); }

void ref_free(ref_csr_out* m) {
    std::free(m->row_ptr);
    std::free(m->col);
    std::free(m->val);
    m->row_ptr = nullptr;
    m->col = nullptr;
    m->val = nullptr;
}

int ref_serial_spgemm(const ref_csr* a, const ref_csr* b, ref_csr_out* out) {
    return guard([&] { from_matrix(serialSpgemm(to_matrix(a), to_matrix(b)), out); });
}

int ref_scalar_multiplication_count(const ref_csr* a, const ref_csr* b, int64_t* out) {
    return guard([&] { *out = scalarMultiplicationCount(to_matrix(a), to_matrix(b)); });
}

// The baseline local multiply with all of B local and no halo rows.
int ref_spgemm(const ref_csr* a, const ref_csr* b, int threads, int chunk, ref_csr_out* out) {
    return guard([&] {
        const CsrMatrix ma = to_matrix(a), mb = to_matrix(b);
        if (threads > 0) omp_set_num_threads(threads);
        omp_set_schedule(omp_sched_guided, chunk > 0 ? chunk : 64);
        RemoteSparseRows none = makeRemoteSparseRows(RemoteRowPlan{});
        from_matrix(spgemm(ma, RowBlock{0, mb.rows}, mb, none, MPI_COMM_WORLD), out);
    });
}

// The baseline multiply timed on caller-owned matrices (no conversion inside
// the timed call); returns the seconds of one spgemm() call.
int ref_spgemm_timed(const ref_csr* a, const ref_csr* b, int threads, int chunk, int repeats,
                     double* seconds, int64_t* nnz) {
    return guard([&] {
        const CsrMatrix ma = to_matrix(a), mb = to_matrix(b);
        if (threads > 0) omp_set_num_threads(threads);
        omp_set_schedule(omp_sched_guided, chunk > 0 ? chunk : 64);
        RemoteSparseRows none = makeRemoteSparseRows(RemoteRowPlan{});
        for (int i = 0; i < repeats; ++i) {
            const double t0 = MPI_Wtime();
            CsrMatrix c = spgemm(ma, RowBlock{0, mb.rows}, mb, none, MPI_COMM_WORLD);
            seconds[i] = MPI_Wtime() - t0;
            *nnz = static_cast<int64_t>(c.values.size());
        }
    });
}

void* ref_accum_create(int32_t rows, int32_t cols) { return new trident::LocalAccumulator(rows, cols); }
void ref_accum_destroy(void* h) { delete static_cast<trident::LocalAccumulator*>(h); }
int ref_accum_add(void* h, const ref_csr* a, const ref_csr* b) {
    return guard([&] { static_cast<trident::LocalAccumulator*>(h)->addProduct(to_matrix(a), to_matrix(b)); });
}
int ref_accum_finish(void* h, ref_csr_out* out) {
    return guard([&] { from_matrix(static_cast<trident::LocalAccumulator*>(h)->finish(), out); });
}

// validateProduct (Full when full != 0, else Partial), uncached.  Its stdout
// diagnostics are suppressed.
int ref_validate(const ref_csr* a, const ref_csr* b, const ref_csr* c, int full, ref_validation* out) {
    return guard([&] {
        std::ostringstream sink;
        auto* old = std::cout.rdbuf(sink.rdbuf());
        ValidationResult v;
        try {
            v = validateProduct(to_matrix(a), to_matrix(b), to_matrix(c),
                                full ? ValidationMode::Full : ValidationMode::Partial);
        } catch (...) {
            std::cout.rdbuf(old);
            throw;
        }
        std::cout.rdbuf(old);
        out->passed = v.passed;
        out->row_nnz_mismatches = v.rowNnzMismatches;
        out->rejected = v.rejectedCoordinates;
        out->max_abs_error = v.maxAbsoluteError ? *v.maxAbsoluteError : __builtin_nan("");
        out->max_error_ratio = static_cast<double>(v.maxErrorRatio);
    });
}

int ref_read_mtx(const char* path, ref_csr_out* out) {
    return guard([&] { from_matrix(readMatrixMarket(path), out); });
}

}  // extern "C"
