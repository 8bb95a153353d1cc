// K1 row-work binning, K1b bin scatter, K3 int64 scan and K5 zero compaction.
//
// K1 computes ub_i = nnz(S_i) + sum_{k in A_i} nnz(B_k), the number of scalar
// products of output row i (scalarMultiplicationCount, spgemm_common.cpp:474-487,
// per row).  It also validates every index it follows: A's row offsets, A's
// columns against B.rows (the reference throws "A contains a column index
// outside B's row range", spgemm_common.cpp:141-143) and the offsets of every
// referenced B row.  HBM traffic: A.rp (8 B/row), A.ci (4 B/entry) and one B.rp
// pair per A entry (16 B/entry).
#include "spg_common.cuh"

namespace spg {
namespace {

constexpr int kRowworkThreads = 256;

__device__ inline int job_of_row(const int64_t* job_row_base, int njobs, int64_t g) {
    int lo = 0, hi = njobs - 1;  // last job with base <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (job_row_base[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(kRowworkThreads)
rowwork_kernel(const Job* __restrict__ jobs, int njobs, const int64_t* __restrict__ job_row_base,
               int64_t total_rows, Stats* __restrict__ stats, ErrWord* __restrict__ err) {
    __shared__ unsigned long long s_bins[kNumBins];
    __shared__ unsigned long long s_products, s_max, s_split;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < kNumBins) s_bins[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        s_products = 0;
        s_max = 0;
        s_split = 0;
    }
    __syncthreads();

    const int64_t warps = static_cast<int64_t>(gridDim.x) * (kRowworkThreads / 32);
    for (int64_t g = static_cast<int64_t>(blockIdx.x) * (kRowworkThreads / 32) + (threadIdx.x >> 5);
         g < total_rows; g += warps) {
        const int j = job_of_row(job_row_base, njobs, g);
        const Job& J = jobs[j];
        const int row = static_cast<int>(g - job_row_base[j]);
        const int64_t a0 = J.A.rp[row], a1 = J.A.rp[row + 1];
        bool bad_row = a0 < 0 || a1 < a0 || a1 > J.A.nnz;
        int64_t len = 0;
        if (!bad_row) {
            for (int64_t p = a0 + lane; p < a1; p += 32) {
                const int32_t k = J.A.ci[p];
                if (k < 0 || k >= J.B.rows) {
                    raise_error(err, kErrColumnRange, 1, p);
                    continue;
                }
                const int64_t s = J.B.rp[k], e = J.B.rp[k + 1];
                if (s < 0 || e < s || e > J.B.nnz) {
                    raise_error(err, kErrInvalid, 2, k);
                    continue;
                }
                len += e - s;
            }
        }
        len = warp_sum(len);
        if (lane == 0) {
            if (bad_row) raise_error(err, kErrInvalid, 3, row);
            if (J.S.rp) len += J.S.rp[row + 1] - J.S.rp[row];
            J.ub[row] = len;
            J.cnt[row] = len;  // upper-bound layout; the exact mode's symbolic phase overwrites it
            atomicAdd(&s_bins[bin_of(len)], 1ull);
            atomicAdd(&s_products, static_cast<unsigned long long>(len));
            atomicMax(&s_max, static_cast<unsigned long long>(len));
            if (len > kSplitThreshold) atomicAdd(&s_split, static_cast<unsigned long long>(len));
        }
    }
    __syncthreads();
    if (threadIdx.x < kNumBins && s_bins[threadIdx.x]) atomicAdd(&stats->bin_count[threadIdx.x], s_bins[threadIdx.x]);
    if (threadIdx.x == 0) {
        atomicAdd(&stats->products, s_products);
        atomicMax(&stats->max_ub, s_max);
        if (s_split) atomicAdd(&stats->split_products, s_split);
    }
}

__global__ void bin_offsets_kernel(const Stats* __restrict__ stats, int64_t* __restrict__ bin_off) {
    if (threadIdx.x == 0) {
        int64_t acc = 0;
        for (int b = 0; b < kNumBins; ++b) {
            bin_off[b] = acc;
            if (b != kBinEmpty) acc += static_cast<int64_t>(stats->bin_count[b]);
        }
        bin_off[kNumBins] = acc;
    }
}

__global__ void __launch_bounds__(256)
bin_scatter_kernel(const Job* __restrict__ jobs, int njobs, const int64_t* __restrict__ job_row_base,
                   int64_t total_rows, const int64_t* __restrict__ bin_off,
                   unsigned long long* __restrict__ cursor, int64_t* __restrict__ items) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * blockDim.x; base < total_rows; base += stride) {
        const int64_t g = base + threadIdx.x;
        int b = kBinEmpty;
        int j = 0, row = 0;
        if (g < total_rows) {
            j = job_of_row(job_row_base, njobs, g);
            row = static_cast<int>(g - job_row_base[j]);
            b = bin_of(jobs[j].ub[row]);
        }
        // Warp-aggregated cursor increments: one atomic per distinct bin.
        const unsigned peers = __match_any_sync(0xffffffffu, b);
        const int leader = __ffs(peers) - 1;
        unsigned long long slot = 0;
        if (lane == leader && b != kBinEmpty) slot = atomicAdd(&cursor[b], static_cast<unsigned long long>(__popc(peers)));
        slot = __shfl_sync(0xffffffffu, slot, leader);
        if (b != kBinEmpty) {
            const int rank = __popc(peers & lanemask_lt());
            items[bin_off[b] + static_cast<int64_t>(slot) + rank] = make_item(j, row);
        }
    }
}

// ---------------------------------------------------------------------------
// K3: exclusive int64 scan in three phases (tile sums, scan of the sums, tile
// scans).  No block waits on another block.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ inline int64_t block_excl_scan(int64_t v, int64_t* s_warp, int64_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int64_t incl = warp_incl_scan(v, lane);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < nw ? s_warp[lane] : 0;
        const int64_t wi = warp_incl_scan(w, lane);
        if (lane < nw) s_warp[lane] = wi - w;
        if (lane == nw - 1) s_warp[32] = wi;
    }
    __syncthreads();
    const int64_t out = s_warp[warp] + incl - v;
    total = s_warp[32];
    __syncthreads();
    return out;
}

__global__ void __launch_bounds__(kScanThreads)
scan_reduce_kernel(const int64_t* __restrict__ data, int64_t n, int64_t* __restrict__ partials) {
    __shared__ int64_t s_warp[33];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile;
    int64_t sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t idx = base + i * kScanThreads + threadIdx.x;
        if (idx < n) sum += data[idx];
    }
    int64_t total;
    block_excl_scan(sum, s_warp, total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024)
scan_partials_kernel(int64_t* __restrict__ partials, int64_t nparts, int64_t* __restrict__ grand_total) {
    __shared__ int64_t s_warp[33];
    int64_t carry = 0;
    for (int64_t base = 0; base < nparts; base += blockDim.x) {
        const int64_t idx = base + threadIdx.x;
        const int64_t v = idx < nparts ? partials[idx] : 0;
        int64_t total;
        const int64_t ex = block_excl_scan(v, s_warp, total);
        if (idx < nparts) partials[idx] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *grand_total = carry;
}

__global__ void __launch_bounds__(kScanThreads)
scan_down_kernel(int64_t* __restrict__ data, int64_t n, const int64_t* __restrict__ partials) {
    __shared__ int64_t s_tile[kScanTile];
    __shared__ int64_t s_warp[33];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t idx = base + i * kScanThreads + threadIdx.x;
        s_tile[i * kScanThreads + threadIdx.x] = idx < n ? data[idx] : 0;
    }
    __syncthreads();
    int64_t loc[kScanItems];
    int64_t sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        loc[i] = sum;
        sum += s_tile[threadIdx.x * kScanItems + i];
    }
    int64_t total;
    const int64_t ex = block_excl_scan(sum, s_warp, total) + partials[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) s_tile[threadIdx.x * kScanItems + i] = ex + loc[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t idx = base + i * kScanThreads + threadIdx.x;
        if (idx < n) data[idx] = s_tile[i * kScanThreads + threadIdx.x];
    }
}

// K5: warp per row, copies the stored entries of a row from its C_tmp offset
// (job.cnt, scanned) to its final offset (job.nz, scanned).
__global__ void __launch_bounds__(256)
compact_kernel(const Job* __restrict__ job, int rows, int32_t* __restrict__ out_col, double* __restrict__ out_val) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
        const int64_t src = job->cnt[r], n = job->nz[r + 1] - job->nz[r];
        int32_t* oc = out_col;
        double* ov = out_val;
        int64_t dst = job->nz[r];
        if (!oc) {  // the job's own arrays
            oc = job->out_col;
            ov = job->out_val;
            dst -= job->nz[0];
        }
        for (int64_t q = lane; q < n; q += 32) {
            oc[dst + q] = job->c_col[src + q];
            ov[dst + q] = job->c_val[src + q];
        }
    }
}

// K5 for rows written with holes (upper-bound mode): warp per row, the row's
// reserved slots [cnt[r], cnt[r+1]) are read in order and the slots with a
// column >= 0 are packed at the row's final offset nz[r] (ballot + popc).
// Each warp loads its next row's offsets while it copies the current one, and
// issues eight chunks of 32 slots per step (2.70 -> 2.45 ms on the power-law
// workload, 89% of the measured copy bandwidth; either change alone gave < 2%).
__global__ void __launch_bounds__(256)
compact_holes_kernel(const Job* __restrict__ jobs, int njobs, const int64_t* __restrict__ job_row_base,
                     int64_t total_rows, int32_t* __restrict__ out_col, double* __restrict__ out_val) {
    constexpr int kChunks = 8;
    const int lane = threadIdx.x & 31;
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
    int64_t g = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int j = 0;
    int64_t n_src = 0, n_end = 0, n_dst = 0;
    auto load_row = [&](int64_t row) {
        j = job_of_row(job_row_base, njobs, row);
        const int r = static_cast<int>(row - job_row_base[j]);
        n_src = jobs[j].cnt[r];
        n_end = jobs[j].cnt[r + 1];
        n_dst = jobs[j].nz[r] - (out_col ? 0 : jobs[j].nz[0]);  // the job's own arrays start at its first row
    };
    if (g < total_rows) load_row(g);
    for (; g < total_rows; g += warps) {
        const Job& J = jobs[j];
        int32_t* __restrict__ oc = out_col ? out_col : J.out_col;
        double* __restrict__ ov = out_col ? out_val : J.out_val;
        const int64_t src = n_src, end = n_end;
        int64_t dst = n_dst;
        if (g + warps < total_rows) load_row(g + warps);
        // columns and values are loaded together (a hole's value is read and
        // dropped) so the loads do not wait on each other
        for (int64_t q0 = src; q0 < end; q0 += kChunks * 32) {
            int32_t c[kChunks];
            double v[kChunks];
#pragma unroll
            for (int u = 0; u < kChunks; ++u) {
                const int64_t q = q0 + u * 32 + lane;
                c[u] = q < end ? J.c_col[q] : -1;
                v[u] = q < end ? J.c_val[q] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kChunks; ++u) {
                const unsigned m = __ballot_sync(0xffffffffu, c[u] >= 0);
                if (c[u] >= 0) {
                    const int64_t at = dst + __popc(m & lanemask_lt());
                    oc[at] = c[u];
                    ov[at] = v[u];
                }
                dst += __popc(m);
            }
        }
    }
}

__global__ void gather_kernel(const int64_t* __restrict__ src, const int64_t* __restrict__ idx,
                              int64_t* __restrict__ dst, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[idx[i]];
}

// Small device->host reads by a kernel storing into mapped page-locked memory:
// they do not queue on the copy engines behind bulk result copies.
__global__ void readback_kernel(const unsigned long long* __restrict__ src, unsigned long long* dst, int64_t words) {
    for (int64_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
}

__global__ void add_offset_kernel(int64_t* __restrict__ d, int64_t n, int64_t add) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        d[i] += add;
}

// blockIdx.y selects product j: out[base_j + r] = scanned[base_j + r] - scanned[base_j]
// for r <= rows_j, where base_j = job_row_base[j] + j (each product's offsets
// restart at zero; the start stays in device memory).
__global__ void rebase_jobs_kernel(const int64_t* __restrict__ scanned, int64_t* __restrict__ out,
                                   const int64_t* __restrict__ job_row_base) {
    const int j = blockIdx.y;
    const int64_t base = job_row_base[j] + j;
    const int64_t rows = job_row_base[j + 1] - job_row_base[j];
    const int64_t start = scanned[base];
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r <= rows;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[base + r] = scanned[base + r] - start;
}

// One CTA per product: its scalar products, the sum of its rows' ub.
__global__ void job_products_kernel(const Job* __restrict__ jobs, const int64_t* __restrict__ job_row_base,
                                    int64_t* __restrict__ out) {
    __shared__ int64_t s_part[8];
    const int j = blockIdx.x;
    const int64_t rows = job_row_base[j + 1] - job_row_base[j];
    const int64_t* ub = jobs[j].ub;
    int64_t sum = 0;
    for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) sum += ub[r];
    sum = warp_sum(sum);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += s_part[w];
        out[j] = t;
    }
}

// blockIdx.y selects the product; threads stride over its rows + 1 offsets.
__global__ void rebase_kernel(const RebaseItem* __restrict__ items) {
    const RebaseItem it = items[blockIdx.y];
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r <= it.rows;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x)
        it.rp[r] -= it.start;
}

int grid_for(int64_t work, int per_block, int cap) {
    const int64_t g = (work + per_block - 1) / per_block;
    return static_cast<int>(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

void launch_rowwork(const Job* d_jobs, int njobs, const int64_t* d_job_row_base, int64_t total_rows,
                    Stats* d_stats, ErrWord* d_err, cudaStream_t stream) {
    if (total_rows <= 0) return;
    const int grid = grid_for(total_rows, kRowworkThreads / 32, 152 * 16);
    rowwork_kernel<<<grid, kRowworkThreads, 0, stream>>>(d_jobs, njobs, d_job_row_base, total_rows, d_stats, d_err);
}

void launch_bin_scatter(const Job* d_jobs, int njobs, const int64_t* d_job_row_base, int64_t total_rows,
                        const int64_t* d_bin_off, unsigned long long* d_bin_cursor, int64_t* d_items,
                        cudaStream_t stream) {
    // d_bin_off holds kNumBins+1 entries computed here from the histogram in Stats,
    // which immediately precedes it in the caller's workspace layout.
    if (total_rows <= 0) return;
    const int grid = grid_for(total_rows, 256, 152 * 16);
    bin_scatter_kernel<<<grid, 256, 0, stream>>>(d_jobs, njobs, d_job_row_base, total_rows, d_bin_off,
                                                  d_bin_cursor, d_items);
}

void launch_bin_offsets(const Stats* d_stats, int64_t* d_bin_off, cudaStream_t stream) {
    bin_offsets_kernel<<<1, 32, 0, stream>>>(d_stats, d_bin_off);
}

size_t scan_partials_count(int64_t n) { return static_cast<size_t>((n + kScanTile - 1) / kScanTile) + 1; }

void launch_scan(int64_t* d_data, int64_t n, int64_t* d_partials, cudaStream_t stream) {
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 0) {
        cudaMemsetAsync(d_data, 0, sizeof(int64_t), stream);
        return;
    }
    scan_reduce_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, stream>>>(d_data, n, d_partials);
    scan_partials_kernel<<<1, 1024, 0, stream>>>(d_partials, nb, d_data + n);
    scan_down_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, stream>>>(d_data, n, d_partials);
}

void launch_compact(const Job* d_job, int rows, int32_t* out_col, double* out_val, cudaStream_t stream) {
    if (rows <= 0) return;
    compact_kernel<<<grid_for(rows, 8, 152 * 16), 256, 0, stream>>>(d_job, rows, out_col, out_val);
}

void launch_compact_holes(const Job* d_jobs, int njobs, const int64_t* d_job_row_base, int64_t total_rows,
                          int32_t* out_col, double* out_val, cudaStream_t stream) {
    if (total_rows <= 0) return;
    compact_holes_kernel<<<grid_for(total_rows, 8, 152 * 32), 256, 0, stream>>>(d_jobs, njobs, d_job_row_base,
                                                                              total_rows, out_col, out_val);
}

void launch_gather(const int64_t* d_src, const int64_t* d_idx, int64_t* d_dst, int n, cudaStream_t stream) {
    if (n <= 0) return;
    gather_kernel<<<grid_for(n, 256, 1024), 256, 0, stream>>>(d_src, d_idx, d_dst, n);
}

void launch_job_products(const Job* d_jobs, int njobs, const int64_t* d_job_row_base, int64_t* d_out,
                         cudaStream_t stream) {
    if (njobs <= 0) return;
    job_products_kernel<<<njobs, 256, 0, stream>>>(d_jobs, d_job_row_base, d_out);
}

namespace {

// Split points of `rows` rows into `parts` contiguous blocks of about equal
// scalar products: first[k] is the first row whose preceding products reach
// floor(k * total / parts) (prefix: exclusive scan of the per-row products,
// prefix[rows] = total); first[0] = 0, first[parts] = rows.  With no products
// at all the rows are split by count, as the reference's partitionRows does.
__global__ void partition_kernel(const int64_t* __restrict__ prefix, int64_t rows, int32_t parts,
                                 int32_t* __restrict__ first) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > parts) return;
    const int64_t total = prefix[rows];
    int64_t r;
    if (k == 0) {
        r = 0;
    } else if (k == parts) {
        r = rows;
    } else if (total == 0) {
        r = rows * k / parts;
    } else {
        const int64_t target = static_cast<int64_t>(static_cast<unsigned __int128>(total) * k / parts);
        int64_t lo = 0, hi = rows;  // smallest i with prefix[i] >= target
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (prefix[mid] >= target) hi = mid;
            else lo = mid + 1;
        }
        r = lo;
    }
    first[k] = static_cast<int32_t>(r);
}

}  // namespace

void launch_partition(const int64_t* d_prefix, int64_t rows, int32_t parts, int32_t* d_first, cudaStream_t stream) {
    partition_kernel<<<(parts + 1 + 127) / 128, 128, 0, stream>>>(d_prefix, rows, parts, d_first);
}

void launch_readback(const void* d_src, void* h_dst, size_t bytes, cudaStream_t stream) {
    if (bytes == 0) return;
    readback_kernel<<<1, 256, 0, stream>>>(static_cast<const unsigned long long*>(d_src),
                                           static_cast<unsigned long long*>(h_dst), static_cast<int64_t>(bytes / 8));
}

void launch_rebase_jobs(const int64_t* d_scanned, int64_t* d_out, const int64_t* d_job_row_base, int njobs,
                        int64_t max_rows, cudaStream_t stream) {
    if (njobs <= 0) return;
    const dim3 grid(grid_for(max_rows + 1, 256, 64), static_cast<unsigned>(njobs));
    rebase_jobs_kernel<<<grid, 256, 0, stream>>>(d_scanned, d_out, d_job_row_base);
}

void launch_add_offset(int64_t* d, int64_t n, int64_t add, cudaStream_t stream) {
    if (n <= 0 || add == 0) return;
    add_offset_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, stream>>>(d, n, add);
}

void launch_rebase(const RebaseItem* d_items, int n, int64_t max_rows, cudaStream_t stream) {
    if (n <= 0) return;
    const dim3 grid(grid_for(max_rows + 1, 256, 64), static_cast<unsigned>(n));
    rebase_kernel<<<grid, 256, 0, stream>>>(d_items);
}

}  // namespace spg
