// Shared definitions of the GB300 SpGEMM engine (device side and launchers).
//
// The engine computes C = S + A*B row by row (S is an optional addend used by
// the accumulate mode; a plain product has no S).  Every output coordinate is
// the sequential FP64 sum of its products in the reference's order: the S entry
// first, then A entries in stored order, then B entries in stored order, each
// product rounded once (__dmul_rn) and added with one rounding (__dadd_rn).
// This is the traversal of serialSpgemm (spgemm_common.cpp:131-178) and of the
// baseline spgemm() row loop (spgemm_exchange.cpp:279-309), so results are
// bit-identical to the reference's serial product.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace spg {

constexpr int kWarp = 32;

// Read-only CSR view in device memory (int64 row offsets, int32 columns, FP64).
struct CsrView {
    int32_t rows = 0, cols = 0;
    int64_t nnz = 0;
    const int64_t* rp = nullptr;
    const int32_t* ci = nullptr;
    const double* v = nullptr;
};

// One product of a launch.  Batched launches carry many jobs; every work item
// names a job and a row.
struct Job {
    CsrView A, B, S;          // S.rp == nullptr: no addend
    int64_t* ub = nullptr;    // [A.rows]  products per row (upper bound of its nnz)
    int64_t* cnt = nullptr;   // [A.rows+1] reserved entries per row (ub, or distinct columns in the
                              // exact mode), scanned in place into C_tmp offsets
    int64_t* nz = nullptr;    // [A.rows+1] stored (nonzero) entries per row
    int32_t* c_col = nullptr; // C_tmp columns (size = total of cnt)
    double* c_val = nullptr;  // C_tmp values
    int64_t row_base = 0;     // first flattened row of this job in a batch
    int32_t holes = 0;        // 1: rows are written slot by slot into their reserved C_tmp range,
                              // column -1 marking unused slots (upper-bound mode); 0: compacted
    int32_t* out_col = nullptr;  // this product's own result arrays (a batch): K5 writes row r at
    double* out_val = nullptr;   // nz[r] - nz[0]; else K5 writes into the arrays it is given
};

// Row bins by product count (ub): capacities 32, 64, then two per power of two
// (3/4 of it and all of it) up to 16384, so that a row fills on average ~85%
// of its bin's slots.  Bin b covers (capacity(b-1), capacity(b)].
//   bins 1-8   warp per row (1, 2, 3, 4, 6, 8, 12, 16 items per lane):
//              <= 32, 64, 96, 128, 192, 256, 384, 512 products
//   bins 9-16  CTA per row, everything in shared memory:
//              <= 768, 1024, 1536, 2048, 3072, 4096, 6144, 8192
//   bins 17-18 CTA per row, product values in a global slab: <= 12288, 16384
//   bin 19     heavier rows: CTA per row, sort in global memory
// In the upper-bound layout the rows of bins 17-19 (more than kSplitThreshold
// products) are split by column range into pieces instead (k_numeric.cu).
constexpr int kBinEmpty = 0;
constexpr int kLastWarpBin = 8;     // capacity 512
constexpr int kLastSmemBin = 16;    // capacity 8192
constexpr int kBinHeavy = 19;
constexpr int kNumBins = 20;
constexpr int64_t kHeavyThreshold = 16384;
constexpr int64_t kSplitThreshold = 8192;

__host__ __device__ inline int clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
    return __clzll(static_cast<long long>(x));
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// Bin of a row with ub scalar products (0 for ub == 0).
__host__ __device__ inline int bin_of(int64_t ub) {
    if (ub <= 0) return kBinEmpty;
    if (ub > kHeavyThreshold) return kBinHeavy;
    if (ub <= 32) return 1;
    if (ub <= 64) return 2;
    const int b = 64 - clz64(static_cast<unsigned long long>(ub - 1));  // ceil(log2 ub), 7..14
    return 2 * (b - 7) + 3 + (ub > (int64_t{3} << (b - 2)) ? 1 : 0);
}

// Largest product count of a bin (its capacity).
__host__ __device__ inline int64_t bin_capacity(int b) {
    if (b == kBinEmpty) return 0;
    if (b == kBinHeavy) return INT64_MAX;
    if (b <= 2) return int64_t{32} << (b - 1);
    const int e = (b - 3) / 2 + 7;  // power of two of the bin pair
    return (b - 3) % 2 == 0 ? (int64_t{3} << (e - 2)) : (int64_t{1} << e);
}

// Error word written by kernels (first error wins) and read by the host at
// each synchronisation point.
struct ErrWord {
    int32_t code;    // spg_status value, 0 = none
    int32_t where;   // kernel tag
    int64_t detail;  // offending row / entry / value
};

enum ErrCode : int32_t {
    kErrNone = 0,
    kErrInvalid = 1,        // malformed CSR or column outside the matrix
    kErrOverflow = 2,       // a count that does not fit
    kErrColumnRange = 3,    // A column outside B's rows
};

// Device-side counters collected per launch (reset by the host).
struct Stats {
    unsigned long long products;      // sum of ub over all rows (the FLOP count / 2)
    unsigned long long max_ub;        // largest ub
    unsigned long long bin_count[kNumBins];
    unsigned long long sym_total;     // sum of cnt
    unsigned long long nz_total;      // sum of nz
    unsigned long long split_products;  // sum of ub over rows of more than kSplitThreshold products
    // the row queue of each bin's numeric launch: rows (or, for the split rows
    // of bins 17-19, pieces) handed out past the launch's first wave
    unsigned long long ticket[kNumBins];
};

// The rows of more than kSplitThreshold products of a call: their scalar
// products (Stats::split_products) and their number (bins 17-19).
struct SplitTotals {
    int64_t products = 0;
    int64_t rows = 0;
};

__device__ inline void raise_error(ErrWord* e, int32_t code, int32_t where, int64_t detail) {
    if (atomicCAS(&e->code, 0, code) == 0) {
        e->where = where;
        e->detail = detail;
    }
}

__device__ inline unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename T>
__device__ inline T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ inline T warp_min(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}

template <typename T>
__device__ inline T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// Inclusive warp scan.
template <typename T>
__device__ inline T warp_incl_scan(T v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T w = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += w;
    }
    return v;
}

// Work item: job index in the high 32 bits, row in the low 32 bits.
__host__ __device__ inline int64_t make_item(int job, int row) {
    return (static_cast<int64_t>(job) << 32) | static_cast<uint32_t>(row);
}
__host__ __device__ inline int item_job(int64_t it) { return static_cast<int>(it >> 32); }
__host__ __device__ inline int item_row(int64_t it) { return static_cast<int>(it & 0xffffffff); }

// --------------------------------------------------------------------------
// Host-side launchers (one per phase).  All are asynchronous on `stream`.

// K1: products per row (ub), bin histogram, product total and input checks.
// Rows of all jobs are flattened: job j owns rows [row_base_j, row_base_j + A_j.rows).
void launch_rowwork(const Job* d_jobs, int njobs, const int64_t* d_job_row_base, int64_t total_rows,
                    Stats* d_stats, ErrWord* d_err, cudaStream_t stream);
// K1b: scatter work items into per-bin lists (d_bin_off from the bin histogram).
void launch_bin_scatter(const Job* d_jobs, int njobs, const int64_t* d_job_row_base, int64_t total_rows,
                        const int64_t* d_bin_off, unsigned long long* d_bin_cursor, int64_t* d_items,
                        cudaStream_t stream);
// K2: distinct columns per row into job.cnt[row] for the items of one bin.
void launch_symbolic(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, int64_t max_ub,
                     void* d_scratch, size_t scratch_bytes, Stats* d_stats, ErrWord* d_err,
                     cudaStream_t stream, int num_sms);
// Global scratch of the symbolic phase (hash slabs of rows above 8192 products).
size_t symbolic_scratch_bytes(const int64_t* bin_count, int64_t max_ub, int num_sms);
// K3: exclusive scan of n+1 int64 counts in place (last entry becomes the total).
void launch_scan(int64_t* d_data, int64_t n, int64_t* d_partials, cudaStream_t stream);
size_t scan_partials_count(int64_t n);
// K4: sorted, summed, zero-free rows into job.c_col/c_val and job.nz[row].
// holes: upper-bound layout (rows above kSplitThreshold products are then
// split into column-range pieces; in the exact layout they keep their CTA
// kernels and the global-slab sort).  split: the call's totals of those rows
// (they size the staging of split rows).  variant: 0 the default team shape of
// the bin, 1 its alternative (where the bin has one; see launch_numeric_alt).
void launch_numeric(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, int64_t max_ub,
                    const SplitTotals& split, void* d_scratch, size_t scratch_bytes, Stats* d_stats, ErrWord* d_err,
                    cudaStream_t stream, int num_sms, bool holes, int variant = 0);
// The alternative shape of a bin; false if the bin has none.
bool launch_numeric_alt(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, Stats* d_stats,
                        ErrWord* d_err, cudaStream_t stream, int num_sms);
constexpr int kNumVariants = 2;
// K4 for the warp-per-row bins (1..kLastWarpBin), compiled separately.
void launch_numeric_warp(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, Stats* d_stats,
                         ErrWord* d_err, cudaStream_t stream, int num_sms);
// Global scratch of the numeric phase: value slabs of the CTA bins, and for
// the rows above 8192 products the staging and pieces of split rows (upper-
// bound layout) or the slabs of their CTA kernels and global-slab sort.
size_t numeric_scratch_bytes(const int64_t* bin_count, int64_t max_ub, const SplitTotals& split, int num_sms,
                             bool holes, bool concurrent = true);
// Totals of the split rows from the row-work statistics.
inline SplitTotals split_totals(const Stats& st) {
    return SplitTotals{static_cast<int64_t>(st.split_products),
                       static_cast<int64_t>(st.bin_count[17] + st.bin_count[18] + st.bin_count[kBinHeavy])};
}
// K5: move rows from C_tmp (offsets job.cnt) to C (offsets job.nz, scanned);
// with out_col == nullptr, into the job's own arrays (Job::out_col / out_val).
void launch_compact(const Job* d_job, int rows, int32_t* out_col, double* out_val, cudaStream_t stream);
// K5 for rows written with holes: keeps the slots whose column is >= 0.
void launch_compact_holes(const Job* d_jobs, int njobs, const int64_t* d_job_row_base, int64_t total_rows,
                          int32_t* out_col, double* out_val, cudaStream_t stream);
// Bin list offsets from the bin histogram.
void launch_bin_offsets(const Stats* d_stats, int64_t* d_bin_off, cudaStream_t stream);

// Batched results: dst[i] = src[idx[i]] and per-product offset rebasing.
struct RebaseItem {
    int64_t* rp;     // rows + 1 offsets of one product
    int64_t start;   // subtracted from every offset
    int64_t rows;
};
void launch_gather(const int64_t* d_src, const int64_t* d_idx, int64_t* d_dst, int n, cudaStream_t stream);
void launch_rebase(const RebaseItem* d_items, int n, int64_t max_rows, cudaStream_t stream);
// GPU validator (k_validate.cu).
size_t validate_cell_bytes();
int validate_hist_buckets();
// flag[0] = 1 if M is malformed (offsets, column range, ordered: strictly
// increasing columns, finite: finite values).
void launch_validate_csr(const CsrView& M, bool ordered, int* d_flag, cudaStream_t st, bool finite = true);
// CSR transpose (k_transpose.cu): A^T's rows keep A's row-major order.
size_t transpose_scratch_bytes(int64_t nnz, int32_t cols);
void launch_transpose(const int64_t* rp, const int32_t* col, const double* val, int32_t rows, int32_t cols, int64_t nnz,
                      int64_t* out_rp, int32_t* out_col, double* out_val, void* scratch, cudaStream_t st);
void launch_validate_slots(const CsrView& A, const CsrView& B, int64_t* d_slots, cudaStream_t st);
void launch_validate_rows(const CsrView& A, const CsrView& B, const CsrView& C, int32_t row0, int32_t row1,
                          const int64_t* d_slot_off, void* d_table, unsigned long long* d_counters,
                          double* d_maxima, unsigned long long* d_hist, cudaStream_t st);
// Copies `bytes` (a multiple of 8, 8-byte aligned) from device memory into
// page-locked host memory with a kernel (no copy engine involved).
void launch_readback(const void* d_src, void* h_dst, size_t bytes, cudaStream_t stream);
// Per-product row offsets restarting at zero, from offsets scanned across a
// batch (product j's rows + 1 entries start at job_row_base[j] + j in both).
void launch_rebase_jobs(const int64_t* d_scanned, int64_t* d_out, const int64_t* d_job_row_base, int njobs,
                        int64_t max_rows, cudaStream_t stream);
// Row blocks of about equal scalar products (spg_partition_rows): d_first
// (parts + 1 entries) from the exclusive scan of the per-row products.
void launch_partition(const int64_t* d_prefix, int64_t rows, int32_t parts, int32_t* d_first, cudaStream_t stream);
// d[i] += add for i < n.
void launch_add_offset(int64_t* d, int64_t n, int64_t add, cudaStream_t stream);
// Scalar products of every product of a batch (after K1): out[j] = sum of job j's ub.
void launch_job_products(const Job* d_jobs, int njobs, const int64_t* d_job_row_base, int64_t* d_out,
                         cudaStream_t stream);

}  // namespace spg
