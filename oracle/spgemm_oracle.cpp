// CPU oracle for the local CSR x CSR product.  TEST INFRASTRUCTURE ONLY.
//
// This file is the checker, never the product: only tests/, the smoke entry
// point and the CPU-baseline leg of bench.py load it.  It restates, in plain
// C++17 + OpenMP, the reference algorithms of malchioman/SpGEMM-hpc-thesis for
// the local multiply and its two validation oracles.  Every function cites the
// reference file:line it follows.  Parity of this restatement is pinned against
// the reference's own sources (oracle/_ref, built by build_ref() in oracle/build.py) and
// against the golden vectors under tests/golden/.
//
// Numerics: compiled with -ffp-contract=off so that `product = a*b; acc += product`
// keeps the separately rounded multiply and add of the reference source on every
// host (GCC contracts a*b+c into an FMA on aarch64 by default).
#include <algorithm>
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

typedef struct {
    int32_t rows, cols;
    int64_t nnz;
    const int64_t* row_ptr;
    const int32_t* col;
    const double* val;
} orc_csr;

typedef struct {
    int32_t rows, cols;
    int64_t nnz;
    int64_t* row_ptr;
    int32_t* col;
    double* val;
} orc_csr_out;

typedef struct {
    int32_t passed;               // rejected == 0 and environment/matrices valid
    int32_t environment_ok;
    int32_t matrices_ok;
    int32_t pad;
    int64_t rejected;             // coordinates whose error exceeds the bound
    int64_t row_nnz_mismatches;   // rows whose stored count differs from the serial count
    int64_t support_mismatches;   // coordinates stored in exactly one of result/serial
    int64_t reference_nnz;        // nonzero serial coordinates in the checked rows
    int64_t checked_coordinates;  // union coordinates walked
    double max_abs_error;         // |c - serial| maximum (the reference's historical field)
    double max_error_ratio;       // max (|c - ref| / bound), rounded up
    double max_rel_error;         // max |c - ref| / |ref| over stored coordinates
    double median_rel_error;      // median of the same
} orc_full_report;

enum { ORC_OK = 0, ORC_INVALID_ARGUMENT = 1, ORC_OVERFLOW = 2, ORC_RUNTIME_ERROR = 3 };

}  // extern "C"

namespace {

thread_local std::string g_last_error;

int fail_with(int code, const std::string& message) {
    g_last_error = message;
    return code;
}

// Overflow-checked int64 sum, as csr_matrix.hpp:20-26 (checkedCsrAdd).
int64_t checked_add(int64_t a, int64_t b, const char* context) {
    if (a < 0 || b < 0 || a > std::numeric_limits<int64_t>::max() - b)
        throw std::overflow_error(std::string(context) + ": invalid/overflowing count");
    return a + b;
}

struct Csr {  // owning result under construction
    int32_t rows = 0, cols = 0;
    std::vector<int64_t> row_ptr;
    std::vector<int32_t> col;
    std::vector<double> val;
};

void export_csr(Csr&& c, orc_csr_out* out) {
    out->rows = c.rows;
    out->cols = c.cols;
    out->nnz = static_cast<int64_t>(c.val.size());
    out->row_ptr = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * c.row_ptr.size()));
    out->col = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max<size_t>(1, c.col.size())));
    out->val = static_cast<double*>(std::malloc(sizeof(double) * std::max<size_t>(1, c.val.size())));
    if (!out->row_ptr || !out->col || !out->val) throw std::bad_alloc();
    std::memcpy(out->row_ptr, c.row_ptr.data(), sizeof(int64_t) * c.row_ptr.size());
    if (!c.col.empty()) std::memcpy(out->col, c.col.data(), sizeof(int32_t) * c.col.size());
    if (!c.val.empty()) std::memcpy(out->val, c.val.data(), sizeof(double) * c.val.size());
}

// A.cols == B.rows, as spgemm_common.cpp:106-110 (validateMultiplicationDimensions).
void require_product_shapes(const orc_csr& a, const orc_csr& b) {
    if (a.cols != b.rows) throw std::invalid_argument("SpGEMM requires A.cols == B.rows");
}

// Ordered accumulation of one output row: A entries in stored order, then B
// entries in stored order; the first product of a column is stored as is and
// later ones are added with a separately rounded add.  This is the traversal
// of forEachSerialProductRow (spgemm_common.cpp:131-156) and of the baseline
// row loop (spgemm_exchange.cpp:279-295).  Returns the touched columns in first
// touch order.
template <bool kCheckRange>
void accumulate_row(const orc_csr& a, const orc_csr& b, int32_t row,
                    std::unordered_map<int32_t, double>& acc, std::vector<int32_t>& touched) {
    acc.clear();
    touched.clear();
    for (int64_t p = a.row_ptr[row]; p < a.row_ptr[row + 1]; ++p) {
        const int32_t k = a.col[p];
        if (kCheckRange && (k < 0 || k >= b.rows))
            throw std::runtime_error("A contains a column index outside B's row range");
        const double av = a.val[p];
        for (int64_t q = b.row_ptr[k]; q < b.row_ptr[k + 1]; ++q) {
            const double product = av * b.val[q];
            auto [slot, fresh] = acc.emplace(b.col[q], product);
            if (fresh) touched.push_back(b.col[q]);
            else slot->second += product;
        }
    }
}

// Sorted nonzero columns of an accumulated row (spgemm_common.cpp:165-176;
// spgemm_exchange.cpp:297-308): exact zeros (+0.0 and -0.0) are dropped,
// NaN and infinities are kept because they compare unequal to zero.
void emit_row(const std::unordered_map<int32_t, double>& acc, std::vector<int32_t>& touched,
              std::vector<int32_t>& cols, std::vector<double>& vals) {
    std::sort(touched.begin(), touched.end());
    for (int32_t c : touched) {
        const double v = acc.at(c);
        if (v != 0.0) {
            cols.push_back(c);
            vals.push_back(v);
        }
    }
}

template <typename F>
int guarded(F&& body) {
    try {
        body();
        return ORC_OK;
    } catch (const std::invalid_argument& e) {
        return fail_with(ORC_INVALID_ARGUMENT, e.what());
    } catch (const std::overflow_error& e) {
        return fail_with(ORC_OVERFLOW, e.what());
    } catch (const std::exception& e) {
        return fail_with(ORC_RUNTIME_ERROR, e.what());
    }
}

// ---------------------------------------------------------------------------
// Full-mode roundoff bound (spgemm_common.cpp:591-675).  For a coordinate with
// m contributing products the double-precision sequential sum obeys
//   |fl(dot) - dot| <= gamma_(2m) * sum|a*b| + 2m*eta / (1 - 2m*u)
// with u the unit roundoff and eta the smallest subnormal; every step of the
// bound itself is rounded upward.
typedef long double ld;

ld round_up(ld x) { return std::nextafter(x, std::numeric_limits<ld>::infinity()); }
ld add_up(ld x, ld y) { return x == 0 ? y : (y == 0 ? x : round_up(x + y)); }
ld mul_up(ld x, ld y) { return (x == 0 || y == 0) ? 0 : round_up(x * y); }
ld div_up(ld x, ld y) { return x == 0 ? 0 : round_up(x / y); }

struct Gamma {
    ld gamma;
    ld underflow;
};

template <typename T>
Gamma gamma_of(int64_t terms) {  // spgemm_common.cpp:652-661 (errorModel)
    const ld ops = mul_up(2, static_cast<ld>(terms));
    const ld scaled = mul_up(ops, std::numeric_limits<T>::epsilon() / 2.0L);
    if (!(scaled < 0.5L)) return {1, std::numeric_limits<ld>::infinity()};
    const ld denom = std::nextafter(1 - scaled, 0.0L);
    return {div_up(scaled, denom), div_up(mul_up(ops, std::numeric_limits<T>::denorm_min()), denom)};
}

struct Cell {  // spgemm_common.cpp:640-645 (NumericCell)
    double serial = 0;
    ld reference = 0;
    ld magnitude = 0;
    int64_t terms = 0;
};

ld bound_of(const Cell& c) {  // spgemm_common.cpp:663-675 (coordinateBound)
    if (c.terms == 0) return 0;
    const Gamma cand = gamma_of<double>(c.terms);
    const Gamma refm = gamma_of<ld>(c.terms);
    if (!(cand.gamma < 1 && refm.gamma < 1) || !std::isfinite(c.reference) ||
        !std::isfinite(c.magnitude))
        return std::numeric_limits<ld>::infinity();
    const ld scale = div_up(add_up(c.magnitude, refm.underflow), std::nextafter(1 - refm.gamma, 0.0L));
    return add_up(mul_up(add_up(cand.gamma, refm.gamma), scale), add_up(cand.underflow, refm.underflow));
}

template <typename T>
bool has_gradual_underflow() {
    volatile T tiny_normal = std::numeric_limits<T>::min();
    volatile T half = T(0.5);
    volatile T sub = std::numeric_limits<T>::denorm_min();
    volatile T big = std::numeric_limits<T>::max();
    return tiny_normal * half == std::numeric_limits<T>::min() / T(2) &&
           sub * big == std::numeric_limits<T>::denorm_min() * std::numeric_limits<T>::max();
}

// spgemm_common.cpp:676-693 (fullNumericEnvironment)
bool numeric_environment_ok() {
#if defined(__FAST_MATH__)
    return false;
#endif
    return std::numeric_limits<double>::radix == 2 && std::numeric_limits<ld>::radix == 2 &&
           std::numeric_limits<double>::digits == 53 &&
           std::numeric_limits<ld>::digits >= std::numeric_limits<double>::digits &&
           std::fegetround() == FE_TONEAREST && has_gradual_underflow<double>() &&
           has_gradual_underflow<ld>();
}

// spgemm_common.cpp:621-638 (validNumericCsr)
bool well_formed(const orc_csr& m, bool ordered) {
    if (m.rows < 0 || m.cols < 0 || !m.row_ptr || m.row_ptr[0] != 0 || m.row_ptr[m.rows] != m.nnz)
        return false;
    for (int32_t r = 0; r < m.rows; ++r) {
        const int64_t first = m.row_ptr[r], end = m.row_ptr[r + 1];
        if (first < 0 || end < first || end > m.nnz) return false;
        int32_t prev = -1;
        for (int64_t p = first; p < end; ++p) {
            const int32_t c = m.col[p];
            if (c < 0 || c >= m.cols || (ordered && c <= prev) || !std::isfinite(m.val[p])) return false;
            prev = c;
        }
    }
    return true;
}

struct RefCell {
    int32_t column;
    double serial;
    ld reference;
    ld bound;
};

// spgemm_common.cpp:695-717 (buildFullRow): serial double sum, long double sum,
// long double magnitude and term count per coordinate, sorted by column.
void full_row(const orc_csr& a, const orc_csr& b, int32_t row, std::unordered_map<int32_t, Cell>& acc,
              std::vector<RefCell>& out) {
    acc.clear();
    for (int64_t p = a.row_ptr[row]; p < a.row_ptr[row + 1]; ++p) {
        const int32_t k = a.col[p];
        for (int64_t q = b.row_ptr[k]; q < b.row_ptr[k + 1]; ++q) {
            Cell& c = acc[b.col[q]];
            const double product = a.val[p] * b.val[q];
            const ld precise = static_cast<ld>(a.val[p]) * static_cast<ld>(b.val[q]);
            c.serial += product;
            c.reference += precise;
            c.magnitude += std::fabs(precise);
            c.terms = checked_add(c.terms, 1, "validation contributions");
        }
    }
    out.clear();
    for (const auto& kv : acc) out.push_back({kv.first, kv.second.serial, kv.second.reference, bound_of(kv.second)});
    std::sort(out.begin(), out.end(), [](const RefCell& x, const RefCell& y) { return x.column < y.column; });
}

struct RowStats {
    int64_t rejected = 0, row_mismatch = 0, support = 0, ref_nnz = 0, walked = 0;
    double max_abs = 0;
    ld max_ratio = 0;
    std::vector<double> rel;
};

// One row of validateFullStreaming's merge walk (spgemm_common.cpp:761-823).
void walk_row(const orc_csr& c, int32_t row, const std::vector<RefCell>& cells, RowStats& st) {
    int64_t row_nnz = 0;
    for (const auto& cell : cells) row_nnz += (cell.serial != 0);
    st.ref_nnz += row_nnz;
    int64_t p = c.row_ptr[row];
    const int64_t end = c.row_ptr[row + 1];
    if (end - p != row_nnz) ++st.row_mismatch;
    size_t e = 0;
    const RefCell none{0, 0, 0, 0};
    while (p < end || e < cells.size()) {
        RefCell cell = none;
        double actual = 0;
        bool stored = false;
        if (e == cells.size() || (p < end && c.col[p] < cells[e].column)) {
            actual = c.val[p++];
            stored = true;
        } else {
            cell = cells[e++];
            if (p < end && c.col[p] == cell.column) {
                actual = c.val[p++];
                stored = true;
            }
        }
        ++st.walked;
        if (stored != (cell.serial != 0)) ++st.support;
        double serial_err = std::fabs(actual - cell.serial);
        if (!std::isfinite(serial_err)) serial_err = std::numeric_limits<double>::infinity();
        st.max_abs = std::max(st.max_abs, serial_err);
        const ld diff = std::fabs(static_cast<ld>(actual) - cell.reference);
        const ld err_up = diff == 0 ? 0 : round_up(diff);
        const ld bnd = cell.bound;
        const bool ok = std::isfinite(serial_err) && std::isfinite(err_up) && std::isfinite(bnd) && err_up <= bnd;
        ld ratio;
        if (!std::isfinite(serial_err) || !std::isfinite(err_up) || !std::isfinite(bnd) || (bnd == 0 && diff != 0))
            ratio = std::numeric_limits<ld>::infinity();
        else if (bnd == 0)
            ratio = 0;
        else
            ratio = ok ? std::min(1.0L, div_up(err_up, bnd)) : div_up(err_up, bnd);
        st.max_ratio = std::max(st.max_ratio, ratio);
        if (!ok) ++st.rejected;
        if (stored && cell.reference != 0 && std::isfinite(cell.reference))
            st.rel.push_back(static_cast<double>(diff / std::fabs(cell.reference)));
    }
}

}  // namespace

extern "C" {

const char* orc_last_error(void) { return g_last_error.c_str(); }

void orc_free(orc_csr_out* m) {
    if (!m) return;
    std::free(m->row_ptr);
    std::free(m->col);
    std::free(m->val);
    m->row_ptr = nullptr;
    m->col = nullptr;
    m->val = nullptr;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// serialSpgemm / buildSerialRowWiseProduct (spgemm_common.cpp:158-178, 470-472).
int orc_serial_spgemm(const orc_csr* a, const orc_csr* b, orc_csr_out* out) {
    return guarded([&] {
        require_product_shapes(*a, *b);
        Csr c;
        c.rows = a->rows;
        c.cols = b->cols;
        c.row_ptr.assign(static_cast<size_t>(a->rows) + 1, 0);
        std::unordered_map<int32_t, double> acc;
        std::vector<int32_t> touched;
        for (int32_t r = 0; r < a->rows; ++r) {
            accumulate_row<true>(*a, *b, r, acc, touched);
            emit_row(acc, touched, c.col, c.val);
            c.row_ptr[r + 1] = static_cast<int64_t>(c.val.size());
        }
        export_csr(std::move(c), out);
    });
}

// The serial product restricted to a list of A rows (same per-row traversal);
// output row i is the product row rows[i].  Used to check sampled rows of
// products too large for a full serial pass.
int orc_serial_rows(const orc_csr* a, const orc_csr* b, const int32_t* rows, int32_t n, orc_csr_out* out) {
    return guarded([&] {
        require_product_shapes(*a, *b);
        Csr c;
        c.rows = n;
        c.cols = b->cols;
        c.row_ptr.assign(static_cast<size_t>(n) + 1, 0);
        std::unordered_map<int32_t, double> acc;
        std::vector<int32_t> touched;
        for (int32_t i = 0; i < n; ++i) {
            if (rows[i] < 0 || rows[i] >= a->rows) throw std::invalid_argument("sample row out of range");
            accumulate_row<true>(*a, *b, rows[i], acc, touched);
            emit_row(acc, touched, c.col, c.val);
            c.row_ptr[i + 1] = static_cast<int64_t>(c.val.size());
        }
        export_csr(std::move(c), out);
    });
}

// The baseline local multiply spgemm() of spgemm_exchange.cpp:258-325 with all
// of B local (localBBlock = {0, B.rows}, no halo rows): one hash map per thread,
// rows under `omp for schedule(runtime)`, per-row sorted nonzero lists, then a
// serial checked prefix sum and concatenation.  A missing B row makes the
// reference abort through fail(); here it is reported as ORC_RUNTIME_ERROR.
// threads <= 0 keeps the OpenMP default; schedule is guided with `chunk`
// (the campaign setting guided/64).
int orc_spgemm_omp(const orc_csr* a, const orc_csr* b, int threads, int chunk, orc_csr_out* out) {
    return guarded([&] {
        const int32_t rows = a->rows;
        std::vector<std::vector<int32_t>> cols_by_row(static_cast<size_t>(rows));
        std::vector<std::vector<double>> vals_by_row(static_cast<size_t>(rows));
        int bad = 0;
#ifdef _OPENMP
        if (threads > 0) omp_set_num_threads(threads);
        omp_set_schedule(omp_sched_guided, chunk > 0 ? chunk : 64);
#endif
#pragma omp parallel
        {
            std::unordered_map<int32_t, double> acc;
            std::vector<int32_t> touched;
#pragma omp for schedule(runtime)
            for (int32_t r = 0; r < rows; ++r) {
                acc.clear();
                touched.clear();
                for (int64_t p = a->row_ptr[r]; p < a->row_ptr[r + 1]; ++p) {
                    const int32_t k = a->col[p];
                    if (k < 0 || k >= b->rows) {
#pragma omp atomic write
                        bad = 1;
                        continue;
                    }
                    const double av = a->val[p];
                    for (int64_t q = b->row_ptr[k]; q < b->row_ptr[k + 1]; ++q) {
                        const double product = av * b->val[q];
                        auto [slot, fresh] = acc.emplace(b->col[q], product);
                        if (fresh) touched.push_back(b->col[q]);
                        else slot->second += product;
                    }
                }
                cols_by_row[r].reserve(touched.size());
                vals_by_row[r].reserve(touched.size());
                emit_row(acc, touched, cols_by_row[r], vals_by_row[r]);
            }
        }
        if (bad) throw std::runtime_error("missing a remote sparse row required by A");
        Csr c;
        c.rows = rows;
        c.cols = b->cols;
        c.row_ptr.assign(static_cast<size_t>(rows) + 1, 0);
        int64_t total = 0;
        for (int32_t r = 0; r < rows; ++r) {
            total = checked_add(total, static_cast<int64_t>(vals_by_row[r].size()), "local result prefix");
            c.row_ptr[r + 1] = total;
        }
        c.col.reserve(static_cast<size_t>(total));
        c.val.reserve(static_cast<size_t>(total));
        for (int32_t r = 0; r < rows; ++r) {
            c.col.insert(c.col.end(), cols_by_row[r].begin(), cols_by_row[r].end());
            c.val.insert(c.val.end(), vals_by_row[r].begin(), vals_by_row[r].end());
        }
        export_csr(std::move(c), out);
    });
}

// The same baseline row loop over a contiguous slice of A's rows, discarding
// the result rows after counting them.  It times the reference's hot loop on a
// bounded sample of a large product.  Returns the nonzeros produced.
int orc_spgemm_omp_rows(const orc_csr* a, const orc_csr* b, int32_t first, int32_t count, int threads,
                        int chunk, int64_t* nnz_out) {
    orc_csr slice = *a;
    if (first < 0 || count < 0 || first + count > a->rows) return fail_with(ORC_INVALID_ARGUMENT, "bad slice");
    // A row slice keeps the parent's absolute row offsets; shift the view.
    std::vector<int64_t> rp(static_cast<size_t>(count) + 1);
    for (int32_t i = 0; i <= count; ++i) rp[i] = a->row_ptr[first + i] - a->row_ptr[first];
    slice.rows = count;
    slice.row_ptr = rp.data();
    slice.col = a->col + a->row_ptr[first];
    slice.val = a->val + a->row_ptr[first];
    slice.nnz = rp[count];
    orc_csr_out c{};
    const int rc = orc_spgemm_omp(&slice, b, threads, chunk, &c);
    if (rc == ORC_OK) {
        *nnz_out = c.nnz;
        orc_free(&c);
    }
    return rc;
}

// scalarMultiplicationCount (spgemm_common.cpp:474-487): P = sum over A entries
// of nnz(B row).  The reference's FLOP count is 2P.
int orc_scalar_multiplication_count(const orc_csr* a, const orc_csr* b, int64_t* count) {
    return guarded([&] {
        require_product_shapes(*a, *b);
        int64_t total = 0;
        for (int32_t r = 0; r < a->rows; ++r)
            for (int64_t p = a->row_ptr[r]; p < a->row_ptr[r + 1]; ++p) {
                const int32_t k = a->col[p];
                if (k < 0 || k >= b->rows)
                    throw std::runtime_error("A contains a column index outside B's row range");
                total = checked_add(total, b->row_ptr[k + 1] - b->row_ptr[k], "scalar products");
            }
        *count = total;
    });
}

// buildPartialReference (spgemm_common.cpp:541-554): per-row count of nonzero
// serial sums, plus whether every serial sum is finite.  Rows are independent,
// so they are spread over OpenMP threads; each row uses the serial traversal.
int orc_partial_reference(const orc_csr* a, const orc_csr* b, int64_t* row_nnz, int32_t* finite) {
    return guarded([&] {
        require_product_shapes(*a, *b);
        int all_finite = 1, bad = 0;
#pragma omp parallel
        {
            std::unordered_map<int32_t, double> acc;
            std::vector<int32_t> touched;
#pragma omp for schedule(dynamic, 256) reduction(& : all_finite) reduction(| : bad)
            for (int32_t r = 0; r < a->rows; ++r) {
                try {
                    accumulate_row<true>(*a, *b, r, acc, touched);
                } catch (const std::exception&) {
                    bad |= 1;
                    continue;
                }
                int64_t n = 0;
                for (const auto& kv : acc) {
                    if (!std::isfinite(kv.second)) all_finite &= 0;
                    if (kv.second != 0.0) ++n;
                }
                row_nnz[r] = n;
            }
        }
        if (bad) throw std::runtime_error("A contains a column index outside B's row range");
        *finite = all_finite;
    });
}

// comparePartialReference (spgemm_common.cpp:556-572): shapes, finiteness of
// both sides and the exact stored count of every row.
int orc_compare_partial(const int64_t* row_nnz, int32_t ref_finite, int32_t ref_rows, int32_t ref_cols,
                        const orc_csr* c, int32_t* passed, int64_t* mismatches) {
    return guarded([&] {
        *mismatches = 0;
        if (c->rows != ref_rows || c->cols != ref_cols) {
            *passed = 0;
            return;
        }
        bool ok = ref_finite != 0;
        for (int64_t p = 0; p < c->nnz; ++p)
            if (!std::isfinite(c->val[p])) ok = false;
        int64_t bad = 0;
        for (int32_t r = 0; r < ref_rows; ++r)
            if (row_nnz[r] != c->row_ptr[r + 1] - c->row_ptr[r]) ++bad;
        *mismatches = bad;
        *passed = ok && bad == 0;
    });
}

// validateFullStreaming without a cache (spgemm_common.cpp:720-851), optionally
// restricted to a list of rows (rows == NULL checks every row; then C holds the
// whole product; otherwise C row i is product row rows[i]).  Adds the max and
// median relative error over stored coordinates against the long double sum.
int orc_validate_full(const orc_csr* a, const orc_csr* b, const orc_csr* c, const int32_t* rows, int32_t n,
                      orc_full_report* rep) {
    return guarded([&] {
        std::memset(rep, 0, sizeof(*rep));
        rep->environment_ok = numeric_environment_ok();
        const int32_t nrows = rows ? n : a->rows;
        rep->matrices_ok = well_formed(*a, false) && well_formed(*b, false) && well_formed(*c, true) &&
                           a->cols == b->rows && c->rows == nrows && c->cols == b->cols;
        if (rows)
            for (int32_t i = 0; i < n; ++i)
                if (rows[i] < 0 || rows[i] >= a->rows) rep->matrices_ok = 0;
        rep->max_abs_error = std::numeric_limits<double>::infinity();
        rep->rejected = 1;
        if (!rep->environment_ok || !rep->matrices_ok) return;
        RowStats total;
        int threads = orc_max_threads();
        std::vector<RowStats> per(static_cast<size_t>(threads));
#pragma omp parallel
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            std::unordered_map<int32_t, Cell> acc;
            std::vector<RefCell> cells;
#pragma omp for schedule(dynamic, 64)
            for (int32_t i = 0; i < nrows; ++i) {
                full_row(*a, *b, rows ? rows[i] : i, acc, cells);
                walk_row(*c, i, cells, per[t]);
            }
        }
        for (auto& s : per) {
            total.rejected += s.rejected;
            total.row_mismatch += s.row_mismatch;
            total.support += s.support;
            total.ref_nnz += s.ref_nnz;
            total.walked += s.walked;
            total.max_abs = std::max(total.max_abs, s.max_abs);
            total.max_ratio = std::max(total.max_ratio, s.max_ratio);
            total.rel.insert(total.rel.end(), s.rel.begin(), s.rel.end());
        }
        rep->rejected = total.rejected;
        rep->row_nnz_mismatches = total.row_mismatch;
        rep->support_mismatches = total.support;
        rep->reference_nnz = total.ref_nnz;
        rep->checked_coordinates = total.walked;
        rep->max_abs_error = total.max_abs;
        rep->max_error_ratio = static_cast<double>(total.max_ratio);
        if (!total.rel.empty()) {
            auto mid = total.rel.begin() + static_cast<long>(total.rel.size() / 2);
            std::nth_element(total.rel.begin(), mid, total.rel.end());
            rep->median_rel_error = *mid;
            rep->max_rel_error = *std::max_element(total.rel.begin(), total.rel.end());
        }
        rep->passed = total.rejected == 0;
    });
}

// ---------------------------------------------------------------------------
// trident::LocalAccumulator (matrix_blocks.cpp:152-200): one hash map per output
// row that survives across addProduct calls; `acc[col] += a*b` starts each new
// coordinate from +0.0; exact zeros are removed only in finish().
struct orc_accum {
    int32_t rows, cols;
    std::vector<std::unordered_map<int32_t, double>> maps;
};

void* orc_accum_create(int32_t rows, int32_t cols) {
    if (rows < 0 || cols < 0) return nullptr;
    auto* h = new orc_accum{rows, cols, {}};
    h->maps.resize(static_cast<size_t>(rows));
    return h;
}

void orc_accum_destroy(void* h) { delete static_cast<orc_accum*>(h); }

int orc_accum_add(void* handle, const orc_csr* a, const orc_csr* b) {
    auto* h = static_cast<orc_accum*>(handle);
    return guarded([&] {
        if (a->cols != b->rows || a->rows != h->rows || b->cols != h->cols)
            throw std::invalid_argument("incompatible Trident partial product shapes");
#pragma omp parallel for schedule(dynamic, 64)
        for (int32_t r = 0; r < a->rows; ++r) {
            auto& acc = h->maps[r];
            for (int64_t p = a->row_ptr[r]; p < a->row_ptr[r + 1]; ++p) {
                const int32_t k = a->col[p];
                for (int64_t q = b->row_ptr[k]; q < b->row_ptr[k + 1]; ++q) {
                    const double product = a->val[p] * b->val[q];
                    acc[b->col[q]] += product;
                }
            }
        }
    });
}

int orc_accum_finish(void* handle, orc_csr_out* out) {
    auto* h = static_cast<orc_accum*>(handle);
    return guarded([&] {
        Csr c;
        c.rows = h->rows;
        c.cols = h->cols;
        c.row_ptr.assign(static_cast<size_t>(h->rows) + 1, 0);
        std::vector<std::pair<int32_t, double>> row;
        for (int32_t r = 0; r < h->rows; ++r) {
            row.clear();
            for (const auto& kv : h->maps[r])
                if (kv.second != 0.0) row.push_back(kv);
            std::sort(row.begin(), row.end(),
                      [](const auto& x, const auto& y) { return x.first < y.first; });
            for (const auto& kv : row) {
                c.col.push_back(kv.first);
                c.val.push_back(kv.second);
            }
            c.row_ptr[r + 1] = checked_add(c.row_ptr[r], static_cast<int64_t>(row.size()),
                                           "Trident local result prefix");
        }
        export_csr(std::move(c), out);
    });
}

// ---------------------------------------------------------------------------
// readMatrixMarket (matrix_market.cpp:28-145): coordinate real/integer/pattern,
// general/symmetric/skew-symmetric/hermitian; mirrored entries follow their
// source entry; file order (including duplicates and explicit zeros) is kept
// inside every row; 'D'/'d' exponents are accepted.
int orc_read_mtx(const char* path, orc_csr_out* out) {
    return guarded([&] {
        std::ifstream in(path);
        if (!in) throw std::runtime_error(std::string("cannot open Matrix Market file: ") + path);
        auto lower = [](std::string s) {
            for (auto& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
            return s;
        };
        auto skippable = [](const std::string& line) {
            const size_t f = line.find_first_not_of(" \t\r\n");
            return f == std::string::npos || line[f] == '%';
        };
        std::string line;
        if (!std::getline(in, line)) throw std::runtime_error("Matrix Market file is empty");
        std::istringstream head(line);
        std::string banner, object, storage, field, symmetry, extra;
        head >> banner >> object >> storage >> field >> symmetry;
        object = lower(object);
        storage = lower(storage);
        field = lower(field);
        symmetry = lower(symmetry);
        if (banner != "%%MatrixMarket" || object != "matrix" || storage != "coordinate" || (head >> extra))
            throw std::runtime_error("only Matrix Market coordinate matrices are supported");
        if (field != "real" && field != "integer" && field != "pattern")
            throw std::runtime_error("only real, integer, and pattern fields are supported");
        if (symmetry != "general" && symmetry != "symmetric" && symmetry != "skew-symmetric" &&
            symmetry != "hermitian")
            throw std::runtime_error("unsupported Matrix Market symmetry: " + symmetry);
        do {
            if (!std::getline(in, line)) throw std::runtime_error("Matrix Market file has no size line");
        } while (skippable(line));
        int rows = 0, cols = 0;
        int64_t entries = 0;
        {
            std::istringstream dims(line);
            if (!(dims >> rows >> cols >> entries) || rows <= 0 || cols <= 0 || entries < 0 || (dims >> extra))
                throw std::runtime_error("invalid Matrix Market dimensions");
        }
        const bool mirrored = symmetry != "general";
        if (mirrored && rows != cols)
            throw std::runtime_error("Matrix Market " + symmetry + " storage requires a square matrix");
        struct Entry {
            int32_t r, c;
            double v;
        };
        std::vector<Entry> list;
        list.reserve(static_cast<size_t>(mirrored ? 2 * entries : entries));
        for (int64_t e = 0; e < entries; ++e) {
            do {
                if (!std::getline(in, line)) throw std::runtime_error("unexpected end of Matrix Market entries");
            } while (skippable(line));
            for (auto& ch : line) {
                if (ch == 'D') ch = 'E';
                if (ch == 'd') ch = 'e';
            }
            std::istringstream fields(line);
            int r = 0, c = 0;
            double v = 1.0;
            if (!(fields >> r >> c) || (field != "pattern" && !(fields >> v)) || !std::isfinite(v) ||
                (fields >> extra))
                throw std::runtime_error("invalid Matrix Market entry");
            if (r < 1 || r > rows || c < 1 || c > cols)
                throw std::runtime_error("Matrix Market entry index is out of range");
            --r;
            --c;
            if (symmetry == "skew-symmetric" && r == c && v != 0.0)
                throw std::runtime_error("skew-symmetric diagonal must be zero");
            list.push_back({r, c, v});
            if (mirrored && r != c) list.push_back({c, r, symmetry == "skew-symmetric" ? -v : v});
        }
        while (std::getline(in, line))
            if (!skippable(line)) throw std::runtime_error("more Matrix Market entries than declared");
        Csr m;
        m.rows = rows;
        m.cols = cols;
        m.row_ptr.assign(static_cast<size_t>(rows) + 1, 0);
        for (const auto& e : list) ++m.row_ptr[e.r + 1];
        for (int r = 0; r < rows; ++r) m.row_ptr[r + 1] = checked_add(m.row_ptr[r + 1], m.row_ptr[r], "prefix");
        m.col.resize(list.size());
        m.val.resize(list.size());
        std::vector<int64_t> cursor(m.row_ptr.begin(), m.row_ptr.end() - 1);
        for (const auto& e : list) {
            const int64_t at = cursor[e.r]++;
            m.col[at] = e.c;
            m.val[at] = e.v;
        }
        export_csr(std::move(m), out);
    });
}

}  // extern "C"
