// K2 symbolic phase: the number of distinct columns of every output row.
//
// This is the count of `accumulator.emplace` insertions in the reference row
// loop (spgemm_exchange.cpp:288-293), i.e. an upper bound of the row's stored
// entries before exact zeros are dropped.  Rows are counted in open-addressing
// hash tables of at least twice the row's product count:
//   * rows of <= 32 products: one warp, one product per lane, distinct columns
//     found with __match_any_sync (no table);
//   * rows of <= 512 products: one warp per row, table in shared memory;
//   * rows of <= 16384 products: one CTA per row, table in shared memory;
//   * heavier rows: one CTA per row, table in a global-memory slab per CTA.
// Every launch reserves the tables of its bin's largest row only (a power of
// two >= twice the bin capacity), so that the bins of short rows keep many
// CTAs per SM.  It also rejects B columns outside [0, B.cols).
#include <algorithm>

#include "spg_enum.cuh"

namespace spg {
namespace {

constexpr int kSymWarpThreads = 256;
constexpr int kSymHeavyThreads = 512;
constexpr int kLastSymSmemBin = 18;  // rows of <= 16384 products: shared-memory tables
#ifndef SPG_SYM_B64
#define SPG_SYM_B64 10
#endif
#ifndef SPG_SYM_B128
#define SPG_SYM_B128 12
#endif

// Table slots reserved per row (warp bins) or per CTA (CTA bins) for bin b:
// the power of two >= twice its capacity, at least 64.
int sym_table_slots(int b) {
    int64_t t = 64;
    while (t < 2 * bin_capacity(b)) t *= 2;
    return static_cast<int>(t);
}

__device__ inline bool col_ok(int32_t c, int32_t cols, ErrWord* err) {
    if (c < 0 || c >= cols) {
        raise_error(err, kErrInvalid, 4, c);
        return false;
    }
    return true;
}

// Inserts col; returns 1 if it was not present.
__device__ inline int hash_insert(int32_t* tab, uint32_t mask, int log2t, int32_t col) {
    uint32_t h = hash_slot(col, log2t);
    while (true) {
        const int32_t old = atomicCAS(&tab[h], -1, col);
        if (old == -1) return 1;
        if (old == col) return 0;
        h = (h + 1) & mask;
    }
}

__global__ void __launch_bounds__(kSymWarpThreads)
sym_warp_kernel(const Job* __restrict__ jobs, const int64_t* __restrict__ items, int64_t count, int tiny,
                int wtab, ErrWord* __restrict__ err) {
    extern __shared__ int32_t s_dyn[];  // kSymWarpThreads / 32 tables of wtab slots
    __shared__ SegTab<32, int32_t> s_seg[kSymWarpThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (kSymWarpThreads / 32);
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * (kSymWarpThreads / 32) + w; i < count; i += warps) {
        const int64_t it = items[i];
        const Job& J = jobs[item_job(it)];
        const int row = item_row(it);
        const int64_t ub = J.ub[row];
        int found = 0;
        if (tiny) {
            // <= 32 products: product t goes to lane t; count the first lane of each column group.
            int32_t* stage = s_dyn + w * wtab;
            team_products<32, false, int32_t>(J, row, s_seg[w], nullptr, lane, [&](int32_t seq, int32_t c, double, double) {
                stage[seq] = c;
            });
            __syncwarp();
            const bool valid = lane < ub;
            const int32_t col = valid ? stage[lane] : -1;
            __syncwarp();
            if (valid) col_ok(col, J.B.cols, err);
            const unsigned peers = __match_any_sync(0xffffffffu, valid ? col : -1);
            const bool first = valid && (peers & lanemask_lt()) == 0;
            found = __popc(__ballot_sync(0xffffffffu, first));
        } else {
            const int log2t = max(6, ceil_log2(2 * ub));
            const uint32_t tsize = 1u << log2t, mask = tsize - 1;
            int32_t* tab = s_dyn + w * wtab;
            for (uint32_t s = lane; s < tsize; s += 32) tab[s] = -1;
            __syncwarp();
            int mine = 0;
            team_products<32, false, int32_t>(J, row, s_seg[w], nullptr, lane, [&](int32_t, int32_t c, double, double) {
                if (col_ok(c, J.B.cols, err)) mine += hash_insert(tab, mask, log2t, c);
            });
            found = warp_sum(mine);
            __syncwarp();
        }
        if (lane == 0) J.cnt[row] = found;
    }
}

template <int NT>
__global__ void __launch_bounds__(NT)
sym_block_kernel(const Job* __restrict__ jobs, const int64_t* __restrict__ items, int64_t count,
                 ErrWord* __restrict__ err) {
    extern __shared__ int32_t s_tab[];  // the bin's table slots
    __shared__ SegTab<NT, int32_t> s_seg;
    __shared__ int64_t s_warp[NT / 32 + 1];
    __shared__ int s_found;
    for (int64_t i = blockIdx.x; i < count; i += gridDim.x) {
        const int64_t it = items[i];
        const Job& J = jobs[item_job(it)];
        const int row = item_row(it);
        const int log2t = max(6, ceil_log2(2 * J.ub[row]));
        const uint32_t tsize = 1u << log2t, mask = tsize - 1;
        for (uint32_t s = threadIdx.x; s < tsize; s += NT) s_tab[s] = -1;
        if (threadIdx.x == 0) s_found = 0;
        __syncthreads();
        int mine = 0;
        team_products<NT, false, int32_t>(J, row, s_seg, s_warp, threadIdx.x,
                                                        [&](int32_t, int32_t c, double, double) {
            if (col_ok(c, J.B.cols, err)) mine += hash_insert(s_tab, mask, log2t, c);
        });
        mine = warp_sum(mine);
        if ((threadIdx.x & 31) == 0) atomicAdd(&s_found, mine);
        __syncthreads();
        if (threadIdx.x == 0) J.cnt[row] = s_found;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kSymHeavyThreads)
sym_heavy_kernel(const Job* __restrict__ jobs, const int64_t* __restrict__ items, int64_t count,
                 int32_t* __restrict__ slabs, int64_t slab_slots, ErrWord* __restrict__ err) {
    __shared__ SegTab<kSymHeavyThreads> s_seg;
    __shared__ int64_t s_warp[kSymHeavyThreads / 32 + 1];
    __shared__ unsigned long long s_found;
    int32_t* tab = slabs + static_cast<int64_t>(blockIdx.x) * slab_slots;
    for (int64_t i = blockIdx.x; i < count; i += gridDim.x) {
        const int64_t it = items[i];
        const Job& J = jobs[item_job(it)];
        const int row = item_row(it);
        const int log2t = ceil_log2(2 * J.ub[row]);
        const uint32_t tsize = 1u << log2t, mask = tsize - 1;
        for (uint32_t s = threadIdx.x; s < tsize; s += kSymHeavyThreads) tab[s] = -1;
        if (threadIdx.x == 0) s_found = 0;
        __syncthreads();
        int mine = 0;
        team_products<kSymHeavyThreads, false>(J, row, s_seg, s_warp, threadIdx.x,
                                               [&](int64_t, int32_t c, double, double) {
            if (col_ok(c, J.B.cols, err)) mine += hash_insert(tab, mask, log2t, c);
        });
        mine = warp_sum(mine);
        if ((threadIdx.x & 31) == 0) atomicAdd(&s_found, static_cast<unsigned long long>(mine));
        __syncthreads();
        if (threadIdx.x == 0) J.cnt[row] = static_cast<int64_t>(s_found);
        __syncthreads();
    }
}

int capped_grid(int64_t work, int per_block, int cap) {
    const int64_t g = (work + per_block - 1) / per_block;
    return static_cast<int>(g < 1 ? 1 : (g > cap ? cap : g));
}

int heavy_ctas(int64_t count, int num_sms) { return static_cast<int>(count < num_sms * 2 ? count : num_sms * 2); }

}  // namespace

size_t symbolic_scratch_bytes(const int64_t* bin_count, int64_t max_ub, int num_sms) {
    const int64_t count = bin_count[kBinHeavy];  // the only bin with global-memory tables
    if (count == 0) return 0;
    return static_cast<size_t>(heavy_ctas(count, num_sms)) * (size_t{1} << ceil_log2(2 * max_ub)) * sizeof(int32_t);
}

void launch_symbolic(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, int64_t max_ub,
                     void* d_scratch, size_t, Stats*, ErrWord* d_err, cudaStream_t stream, int num_sms) {
    if (count <= 0) return;
    if (bin <= kLastWarpBin) {
        const int wtab = sym_table_slots(bin);
        const int smem = (kSymWarpThreads / 32) * wtab * static_cast<int>(sizeof(int32_t));
        cudaFuncSetAttribute(sym_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        const int grid = capped_grid(count, kSymWarpThreads / 32, num_sms * 32);
        sym_warp_kernel<<<grid, kSymWarpThreads, smem, stream>>>(d_jobs, d_items, count, bin == 1, wtab, d_err);
    } else if (bin <= kLastSymSmemBin) {
        const int smem = sym_table_slots(bin) * static_cast<int>(sizeof(int32_t));
        auto run = [&](auto kernel, int nt) {
            cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            kernel<<<capped_grid(count, 1, num_sms * (2048 / nt)), nt, smem, stream>>>(d_jobs, d_items, count, d_err);
        };
        // CTA size by row size: 6-12 products per thread on the bins below 4096 products
        if (bin <= SPG_SYM_B64) run(sym_block_kernel<64>, 64);
        else if (bin <= SPG_SYM_B128) run(sym_block_kernel<128>, 128);
        else if (bin <= kLastSmemBin) run(sym_block_kernel<256>, 256);
        else run(sym_block_kernel<512>, 512);
    } else {
        const int grid = heavy_ctas(count, num_sms);
        const int64_t slots = int64_t{1} << ceil_log2(2 * max_ub);
        sym_heavy_kernel<<<grid, kSymHeavyThreads, 0, stream>>>(d_jobs, d_items, count,
                                                               static_cast<int32_t*>(d_scratch), slots, d_err);
    }
}

}  // namespace spg
