// GPU validator of a product C = A * B in the reference's two modes.
//
// Full (validateFullStreaming, spgemm_common.cpp:720-851): every coordinate of
// the exact product is recomputed -- the sequential FP64 sum in the reference's
// order (the `serial` cell), a double-double sum of the exact products (the
// reference uses long double), the double-double sum of their magnitudes and
// the term count (NumericCell, :640-645) -- and C's value must lie within the
// roundoff bound of coordinateBound (:663-675):
//   |c - ref| <= (g(m, u) + g(m, u_ref)) * (sum|ab| + h(m, u_ref)) / (1 - g(m, u_ref)) + h(m, u) + h(m, u_ref)
//   g(m, u) = 2m u / (1 - 2m u),  h(m, u) = 2m eta / (1 - 2m u)
// with u = 2^-53, u_ref = 2^-100 (a margin above the double-double sum's own
// rounding) and eta the smallest subnormal; the bound is evaluated with upward
// rounding.  Partial (comparePartialReference, :541-572): C's row counts must
// equal the counts of nonzero serial sums.
//
// The recomputation is the reference's algorithm itself, independent of the
// engine's sort-based kernels: one thread per output row walks the row's
// products in stored order into an open-addressing table of its own (global
// memory, 2^ceil(log2(2 ub)) cells), exactly as buildFullRow (:695-717) fills
// its hash map; then the row of C is merged against the table.
#include "spg_common.cuh"

namespace spg {
namespace {

struct Cell {
    int32_t key;     // column, -1 empty
    int32_t matched; // a stored entry of C was found for it
    int64_t terms;
    double serial, ref_hi, ref_lo, mag_hi, mag_lo;
};

// Error-free transformations (Knuth's TwoSum; FMA-based TwoProduct) and the
// accurate double-double addition built from them.
__device__ inline void two_sum(double a, double b, double& s, double& e) {
    s = __dadd_rn(a, b);
    const double bb = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

__device__ inline void dd_add(double& hi, double& lo, double bh, double bl) {
    double s, e, t, f;
    two_sum(hi, bh, s, e);
    two_sum(lo, bl, t, f);
    e = __dadd_rn(e, t);
    double s2 = __dadd_rn(s, e);
    e = __dsub_rn(e, __dsub_rn(s2, s));
    e = __dadd_rn(e, f);
    hi = __dadd_rn(s2, e);
    lo = __dsub_rn(e, __dsub_rn(hi, s2));
}

__device__ inline double next_down_pos(double x) {  // x > 0 finite
    return __longlong_as_double(__double_as_longlong(x) - 1);
}

// g(m, u) and h(m, u) of the error model, rounded upward (errorModel, :652-661).
__device__ inline void gamma_of(int64_t terms, double u, double& gamma, double& under) {
    const double ops = __dmul_ru(2.0, static_cast<double>(terms));
    const double scaled = __dmul_ru(ops, u);
    if (!(scaled < 0.5)) {
        gamma = 1.0;
        under = __longlong_as_double(0x7ff0000000000000ll);
        return;
    }
    const double denom = next_down_pos(__dsub_rd(1.0, scaled));
    gamma = __ddiv_ru(scaled, denom);
    under = __ddiv_ru(__dmul_ru(ops, 4.9406564584124654e-324), denom);
}

__device__ inline double bound_of(const Cell& c) {
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    if (c.terms == 0) return 0.0;
    double gc, uc, gr, ur;
    gamma_of(c.terms, 0x1p-53, gc, uc);
    gamma_of(c.terms, 0x1p-100, gr, ur);
    if (!(gc < 1.0 && gr < 1.0) || !isfinite(c.ref_hi) || !isfinite(c.mag_hi)) return inf;
    const double mag = __dadd_ru(c.mag_hi, c.mag_lo);
    const double scale = __ddiv_ru(__dadd_ru(mag, ur), next_down_pos(__dsub_rd(1.0, gr)));
    return __dadd_ru(__dmul_ru(__dadd_ru(gc, gr), scale), __dadd_ru(uc, ur));
}

struct Acc {  // per-thread statistics
    unsigned long long rejected = 0, row_mismatch = 0, support = 0, ref_nnz = 0, walked = 0;
    double max_abs = 0.0, max_ratio = 0.0, max_rel = 0.0;
};

constexpr int kHistBuckets = 1 << 14;  // relative errors by their top 14 bits (exponent + 3 mantissa bits)

__device__ inline void atomic_max_pos(double* p, double v) {  // v >= 0 (or +inf)
    atomicMax(reinterpret_cast<unsigned long long*>(p), static_cast<unsigned long long>(__double_as_longlong(v)));
}

// One walked coordinate (walk_row of the merge in validateFullStreaming).
__device__ inline void visit(const Cell& cell, double actual, bool stored, Acc& acc,
                             unsigned long long* hist) {
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    ++acc.walked;
    if (stored != (cell.serial != 0.0)) ++acc.support;
    double serial_err = fabs(__dsub_rn(actual, cell.serial));
    if (!isfinite(serial_err)) serial_err = inf;
    acc.max_abs = fmax(acc.max_abs, serial_err);
    // |actual - (ref_hi + ref_lo)| rounded upward: the difference as a
    // renormalised double-double (s, t), |t| <= ulp(s) / 2, bounded by |s| + |t|
    double dh, dl, ds, dt;
    two_sum(actual, -cell.ref_hi, dh, dl);
    dl = __dsub_rn(dl, cell.ref_lo);
    two_sum(dh, dl, ds, dt);
    const double err_up = (ds == 0.0 && dt == 0.0) ? 0.0 : __dadd_ru(fabs(ds), fabs(dt));
    const double bnd = bound_of(cell);
    const bool ok = isfinite(serial_err) && isfinite(err_up) && isfinite(bnd) && err_up <= bnd;
    double ratio;
    if (!isfinite(serial_err) || !isfinite(err_up) || !isfinite(bnd) || (bnd == 0.0 && err_up != 0.0)) ratio = inf;
    else if (bnd == 0.0) ratio = 0.0;
    else ratio = ok ? fmin(1.0, __ddiv_ru(err_up, bnd)) : __ddiv_ru(err_up, bnd);
    acc.max_ratio = fmax(acc.max_ratio, ratio);
    if (!ok) ++acc.rejected;
    if (stored && cell.ref_hi != 0.0 && isfinite(cell.ref_hi)) {
        const double rel = __ddiv_rn(fabs(ds), fabs(cell.ref_hi));
        acc.max_rel = fmax(acc.max_rel, rel);
        const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(rel));
        atomicAdd(&hist[bits >> 49], 1ull);  // rel >= 0: the top bits order the values
    }
}

__global__ void validate_rows_kernel(CsrView A, CsrView B, CsrView C, int32_t row0, int32_t row1,
                                     const int64_t* __restrict__ slot_off, Cell* __restrict__ table,
                                     unsigned long long* __restrict__ counters, double* __restrict__ maxima,
                                     unsigned long long* __restrict__ hist) {
    Acc acc;
    const int64_t base = slot_off[row0];
    for (int32_t r = row0 + blockIdx.x * blockDim.x + threadIdx.x; r < row1; r += gridDim.x * blockDim.x) {
        const int64_t s0 = slot_off[r] - base;
        const int64_t S = slot_off[r + 1] - slot_off[r];  // 0 or a power of two >= 2
        Cell* T = table + s0;
        int log2s = 0;
        while ((int64_t{1} << log2s) < S) ++log2s;
        for (int64_t q = 0; q < S; ++q) {
            T[q].key = -1;
            T[q].matched = 0;
        }
        // the row's products in reference order (buildFullRow)
        for (int64_t p = A.rp[r]; p < A.rp[r + 1]; ++p) {
            const int32_t k = A.ci[p];
            const double a = A.v[p];
            for (int64_t q = B.rp[k]; q < B.rp[k + 1]; ++q) {
                const int32_t c = B.ci[q];
                const double b = B.v[q];
                const double prod = __dmul_rn(a, b);
                const double err = __fma_rn(a, b, -prod);
                const double ah = prod < 0.0 ? -prod : prod, al = prod < 0.0 ? -err : err;
                uint32_t h = (static_cast<uint32_t>(c) * 0x9E3779B1u) >> (32 - log2s);
                while (T[h].key != -1 && T[h].key != c) h = (h + 1) & static_cast<uint32_t>(S - 1);
                Cell& cell = T[h];
                if (cell.key == -1) {
                    cell.key = c;
                    cell.terms = 1;
                    cell.serial = prod;
                    cell.ref_hi = prod;
                    cell.ref_lo = err;
                    cell.mag_hi = ah;
                    cell.mag_lo = al;
                } else {
                    cell.terms += 1;
                    cell.serial = __dadd_rn(cell.serial, prod);
                    dd_add(cell.ref_hi, cell.ref_lo, prod, err);
                    dd_add(cell.mag_hi, cell.mag_lo, ah, al);
                }
            }
        }
        // merge with C's row: its stored entries first, then the coordinates it lacks
        int64_t row_nnz = 0;
        for (int64_t p = C.rp[r]; p < C.rp[r + 1]; ++p) {
            const int32_t c = C.ci[p];
            Cell none{};
            none.key = c;
            Cell* hit = nullptr;
            if (S > 0) {
                uint32_t h = (static_cast<uint32_t>(c) * 0x9E3779B1u) >> (32 - log2s);
                for (int64_t probes = 0; probes < S && T[h].key != -1; ++probes) {
                    if (T[h].key == c) {
                        hit = &T[h];
                        break;
                    }
                    h = (h + 1) & static_cast<uint32_t>(S - 1);
                }
            }
            if (hit) hit->matched = 1;
            visit(hit ? *hit : none, C.v[p], true, acc, hist);
        }
        for (int64_t q = 0; q < S; ++q) {
            if (T[q].key == -1) continue;
            if (T[q].serial != 0.0) ++row_nnz;
            if (!T[q].matched) visit(T[q], 0.0, false, acc, hist);
        }
        acc.ref_nnz += static_cast<unsigned long long>(row_nnz);
        if (row_nnz != C.rp[r + 1] - C.rp[r]) ++acc.row_mismatch;
    }
    atomicAdd(&counters[0], acc.rejected);
    atomicAdd(&counters[1], acc.row_mismatch);
    atomicAdd(&counters[2], acc.support);
    atomicAdd(&counters[3], acc.ref_nnz);
    atomicAdd(&counters[4], acc.walked);
    atomic_max_pos(&maxima[0], acc.max_abs);
    atomic_max_pos(&maxima[1], acc.max_ratio);
    atomic_max_pos(&maxima[2], acc.max_rel);
}

// Slots of every row's table: 0 for a row without products, else
// 2^ceil(log2(2 ub)) (the products bound the distinct columns).
__global__ void validate_slots_kernel(CsrView A, CsrView B, int64_t* __restrict__ slots) {
    for (int32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < A.rows; r += gridDim.x * blockDim.x) {
        int64_t ub = 0;
        for (int64_t p = A.rp[r]; p < A.rp[r + 1]; ++p) {
            const int32_t k = A.ci[p];
            ub += B.rp[k + 1] - B.rp[k];
        }
        int64_t s = 0;
        if (ub > 0) {
            s = 2;
            while (s < 2 * ub) s <<= 1;
        }
        slots[r] = s;
    }
}

// validNumericCsr (spgemm_common.cpp:621-638): offsets, column range, finite
// values, and (ordered) strictly increasing columns per row.  flag[0] = 1 on
// any violation.
__global__ void validate_csr_kernel(CsrView M, int ordered, int finite, int* __restrict__ flag) {
    for (int32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < M.rows; r += gridDim.x * blockDim.x) {
        const int64_t first = M.rp[r], end = M.rp[r + 1];
        if ((r == 0 && first != 0) || (r == M.rows - 1 && end != M.nnz) || first < 0 || end < first || end > M.nnz) {
            *flag = 1;
            continue;
        }
        int32_t prev = -1;
        for (int64_t p = first; p < end; ++p) {
            const int32_t c = M.ci[p];
            if (c < 0 || c >= M.cols || (ordered && c <= prev) || (finite && !isfinite(M.v[p]))) {
                *flag = 1;
                break;
            }
            prev = c;
        }
    }
}

int grid_rows(int64_t rows, int threads) {
    const int64_t g = (rows + threads - 1) / threads;
    return static_cast<int>(g < 1 ? 1 : (g > 152 * 32 ? 152 * 32 : g));
}

}  // namespace

size_t validate_cell_bytes() { return sizeof(Cell); }
int validate_hist_buckets() { return kHistBuckets; }

void launch_validate_csr(const CsrView& M, bool ordered, int* d_flag, cudaStream_t st, bool finite) {
    if (M.rows <= 0) return;
    validate_csr_kernel<<<grid_rows(M.rows, 128), 128, 0, st>>>(M, ordered ? 1 : 0, finite ? 1 : 0, d_flag);
}

void launch_validate_slots(const CsrView& A, const CsrView& B, int64_t* d_slots, cudaStream_t st) {
    if (A.rows <= 0) return;
    validate_slots_kernel<<<grid_rows(A.rows, 128), 128, 0, st>>>(A, B, d_slots);
}

void launch_validate_rows(const CsrView& A, const CsrView& B, const CsrView& C, int32_t row0, int32_t row1,
                          const int64_t* d_slot_off, void* d_table, unsigned long long* d_counters,
                          double* d_maxima, unsigned long long* d_hist, cudaStream_t st) {
    if (row1 <= row0) return;
    validate_rows_kernel<<<grid_rows(row1 - row0, 64), 64, 0, st>>>(A, B, C, row0, row1, d_slot_off,
                                                                    static_cast<Cell*>(d_table), d_counters,
                                                                    d_maxima, d_hist);
}

}  // namespace spg
