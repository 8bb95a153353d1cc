// K4 numeric phase: row bins that run one row per CTA, the heavy rows, and the
// bin dispatch (warp bins are compiled in k_numeric_warp.cu).  The per-row
// pipeline is in k_numeric_row.cuh.
#include <algorithm>

#include "k_numeric_row.cuh"

namespace spg {
namespace {

// ---------------------------------------------------------------------------
// Heavy rows: one CTA per row, the sort in a global-memory slab of this CTA.
constexpr int kHeavyW = 16;
constexpr int kHeavyItems = 16;
constexpr int kHeavyThreads = kHeavyW * 32;
constexpr int kHeavyTile = kHeavyThreads * kHeavyItems;

struct HeavySmem {
    SegTab<kHeavyThreads> seg;
    int64_t warp_tmp[kHeavyW + 1];
    uint32_t hist[kHistWords<kHeavyW>];
    uint32_t digit_base[256];
    uint32_t digit_tot[256];
    uint32_t cnt[kHeavyW * kHeavyItems];
    int32_t red[2 * kHeavyW];
    uint32_t out_base;
};

struct HeavySlab {
    uint32_t* keys[2];
    uint32_t* seqs[2];
    double* vals;
};

__device__ inline HeavySlab heavy_slab(void* base, int64_t cap, int cta) {
    // per CTA: vals (8*cap) | keys0 | keys1 | seqs0 | seqs1 (4*cap each)
    unsigned char* p = static_cast<unsigned char*>(base) + static_cast<size_t>(cta) * 24 * static_cast<size_t>(cap);
    HeavySlab s;
    s.vals = reinterpret_cast<double*>(p);
    s.keys[0] = reinterpret_cast<uint32_t*>(p + 8 * cap);
    s.keys[1] = s.keys[0] + cap;
    s.seqs[0] = s.keys[1] + cap;
    s.seqs[1] = s.seqs[0] + cap;
    return s;
}

__global__ void __launch_bounds__(kHeavyThreads)
num_heavy_kernel(const Job* __restrict__ jobs, const int64_t* __restrict__ items, int64_t count, void* slabs,
                 int64_t cap, Stats* __restrict__ stats, ErrWord* __restrict__ err) {
    __shared__ HeavySmem sm;
    const HeavySlab sl = heavy_slab(slabs, cap, blockIdx.x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, tid = threadIdx.x;
    unsigned long long kept_total = 0;
    for (int64_t it_i = blockIdx.x; it_i < count; it_i += gridDim.x) {
        const int64_t it = items[it_i];
        const Job& J = jobs[item_job(it)];
        const int row = item_row(it);
        const int64_t P = J.ub[row];
        const int32_t ncols = J.B.cols;

        int32_t lo = INT32_MAX, hi = INT32_MIN;
        team_products<kHeavyThreads, true>(J, row, sm.seg, sm.warp_tmp, tid,
                                           [&](int64_t seq, int32_t c, double b, double a) {
            if (c < 0 || c >= ncols) {
                raise_error(err, kErrInvalid, 4, c);
                c = 0;
            }
            sl.keys[0][seq] = static_cast<uint32_t>(c);
            sl.seqs[0][seq] = static_cast<uint32_t>(seq);
            sl.vals[seq] = __dmul_rn(a, b);
            lo = min(lo, c);
            hi = max(hi, c);
        });
        lo = warp_min(lo);
        hi = warp_max(hi);
        if (lane == 0) {
            sm.red[warp] = lo;
            sm.red[kHeavyW + warp] = hi;
        }
        __syncthreads();
        lo = sm.red[0];
        hi = sm.red[kHeavyW];
        for (int w = 1; w < kHeavyW; ++w) {
            lo = min(lo, sm.red[w]);
            hi = max(hi, sm.red[kHeavyW + w]);
        }
        __syncthreads();
        const uint32_t cmin = static_cast<uint32_t>(lo);
        const uint32_t range = static_cast<uint32_t>(hi - lo);
        const int nbits = range ? 32 - __clz(range) : 0;
        int cur = 0;
        const int64_t ntiles = (P + kHeavyTile - 1) / kHeavyTile;

        for (int shift = 0; shift < nbits; shift += 8) {
            const uint32_t* kin = sl.keys[cur];
            const uint32_t* sin = sl.seqs[cur];
            uint32_t* kout = sl.keys[cur ^ 1];
            uint32_t* sout = sl.seqs[cur ^ 1];
            // digit totals of the whole row
            if (tid < 256) sm.digit_tot[tid] = 0;
            __syncthreads();
            for (int64_t p = tid; p < P; p += kHeavyThreads)
                atomicAdd(&sm.digit_tot[((kin[p] - cmin) >> shift) & 255u], 1u);
            __syncthreads();
            if (warp == 0) {  // exclusive scan of 256 totals, 8 per lane
                uint32_t v[8], tot = 0;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    v[j] = sm.digit_tot[lane * 8 + j];
                    tot += v[j];
                }
                uint32_t base = warp_incl_scan(tot, lane) - tot;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    sm.digit_base[lane * 8 + j] = base;
                    base += v[j];
                }
            }
            __syncthreads();
            for (int64_t t = 0; t < ntiles; ++t) {
                const int64_t tile0 = t * kHeavyTile;
                uint32_t k[kHeavyItems], s[kHeavyItems], rk[kHeavyItems];
                for (int d = tid; d < kHistWords<kHeavyW>; d += kHeavyThreads) sm.hist[d] = 0;
                __syncthreads();
#pragma unroll
                for (int i = 0; i < kHeavyItems; ++i) {
                    const int64_t pos = tile0 + (warp * kHeavyItems + i) * 32 + lane;
                    const bool valid = pos < P;
                    k[i] = valid ? kin[pos] : 0u;
                    s[i] = valid ? sin[pos] : 0u;
                    const uint32_t d = valid ? (((k[i] - cmin) >> shift) & 255u) : 255u;
                    rk[i] = rank_item(d, &sm.hist[hidx<kHeavyW>(d, warp)], lane);
                }
                __syncthreads();
                if (tid < 256) {  // this tile's count of digit tid
                    uint32_t c = 0;
#pragma unroll
                    for (int w = 0; w < kHeavyW; ++w) c += sm.hist[hidx<kHeavyW>(tid, w)];
                    sm.digit_tot[tid] = c;
                }
                __syncthreads();
                scan_counters<kHeavyW>(sm.hist, sm.warp_tmp);
                __syncthreads();
#pragma unroll
                for (int i = 0; i < kHeavyItems; ++i) {
                    const int64_t pos = tile0 + (warp * kHeavyItems + i) * 32 + lane;
                    if (pos < P) {
                        const uint32_t d = ((k[i] - cmin) >> shift) & 255u;
                        // position among this tile's items of digit d, then the row-wide base
                        const uint32_t within = sm.hist[hidx<kHeavyW>(d, warp)] + rk[i] - sm.hist[hidx<kHeavyW>(d, 0)];
                        const uint32_t dst = sm.digit_base[d] + within;
                        kout[dst] = k[i];
                        sout[dst] = s[i];
                    }
                }
                __syncthreads();
                if (tid < 256) sm.digit_base[tid] += sm.digit_tot[tid];
                __syncthreads();
            }
            cur ^= 1;
        }

        // runs and output, tile by tile
        const uint32_t* keys = sl.keys[cur];
        const uint32_t* seqs = sl.seqs[cur];
        if (tid == 0) sm.out_base = 0;
        __syncthreads();
        const int64_t out0 = J.cnt[row];
        for (int64_t t = 0; t < ntiles; ++t) {
            const int64_t tile0 = t * kHeavyTile;
            double sum[kHeavyItems];
            uint32_t col[kHeavyItems];
            unsigned keepmask[kHeavyItems];
#pragma unroll
            for (int i = 0; i < kHeavyItems; ++i) {
                const int64_t pos = tile0 + (warp * kHeavyItems + i) * 32 + lane;
                bool keep = false;
                sum[i] = 0.0;
                col[i] = 0;
                if (pos < P) {
                    const uint32_t key = keys[pos];
                    if (pos == 0 || keys[pos - 1] != key) {
                        double acc = sl.vals[seqs[pos]];
                        for (int64_t q = pos + 1; q < P && keys[q] == key; ++q) acc = __dadd_rn(acc, sl.vals[seqs[q]]);
                        sum[i] = acc;
                        col[i] = key;
                        keep = acc != 0.0;
                    }
                }
                keepmask[i] = __ballot_sync(0xffffffffu, keep);
                if (lane == 0) sm.cnt[warp * kHeavyItems + i] = __popc(keepmask[i]);
            }
            __syncthreads();
            scan_kept<kHeavyW, kHeavyItems>(sm.cnt, sm.red, warp, lane);
            __syncthreads();
            const int64_t tile_out = out0 + sm.out_base;
#pragma unroll
            for (int i = 0; i < kHeavyItems; ++i) {
                if (keepmask[i] & (1u << lane)) {
                    const int64_t idx = tile_out + sm.cnt[warp * kHeavyItems + i] + __popc(keepmask[i] & lanemask_lt());
                    J.c_col[idx] = static_cast<int32_t>(col[i]);
                    J.c_val[idx] = sum[i];
                }
            }
            __syncthreads();
            if (tid == 0) sm.out_base += static_cast<uint32_t>(sm.red[0]);
            __syncthreads();
        }
        if (J.holes)  // upper-bound mode: the unused tail of the reserved range becomes holes
            for (int64_t q = out0 + sm.out_base + tid; q < out0 + P; q += kHeavyThreads) J.c_col[q] = -1;
        if (tid == 0) {
            J.nz[row] = sm.out_base;
            kept_total += sm.out_base;
        }
        __syncthreads();
    }
    if (tid == 0 && kept_total) atomicAdd(&stats->nz_total, kept_total);
}

int heavy_grid(int64_t count, int num_sms) { return static_cast<int>(count < num_sms ? count : num_sms); }

// Product-value slab of one CTA of the two global-slab bins.
constexpr int64_t slab_cap(int bin) { return bin == 17 ? 16 * 32 * 24 : 16 * 32 * 32; }

}  // namespace

size_t numeric_scratch_bytes(const int64_t* bin_count, int64_t max_ub, int num_sms) {
    size_t need = 0;
    for (int b = kLastSmemBin + 1; b < kBinHeavy; ++b)  // the launches run one after the other
        if (bin_count[b])
            need = std::max(need, static_cast<size_t>(slab_grid(bin_count[b], num_sms)) * slab_cap(b) * sizeof(double));
    if (bin_count[kBinHeavy])
        need = std::max(need, static_cast<size_t>(heavy_grid(bin_count[kBinHeavy], num_sms)) * 24 *
                                  static_cast<size_t>(max_ub));
    return need;
}

void launch_numeric(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, int64_t max_ub,
                    void* d_scratch, size_t, Stats* d_stats, ErrWord* d_err, cudaStream_t st, int num_sms) {
    if (count <= 0) return;
    if (bin <= kLastWarpBin) {
        launch_numeric_warp(bin, d_jobs, d_items, count, d_stats, d_err, st, num_sms);
        return;
    }
    double* slab = static_cast<double*>(d_scratch);
    switch (bin) {
        case 9: run_block<4, 6, 6>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;     // <= 768
        case 10: run_block<4, 8, 6>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;    // <= 1024
        case 11: run_block<8, 6, 3>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;    // <= 1536
        case 12: run_block<8, 8, 3>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;    // <= 2048
        case 13: run_block<8, 12, 2>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;   // <= 3072
        case 14: run_block<8, 16, 2>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;   // <= 4096
        case 15: run_block<16, 12, 1>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;  // <= 6144
        case 16: run_block<16, 16, 1>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;  // <= 8192
        case 17: run_block<16, 24, 1, false>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, slab); break;
        case 18: run_block<16, 32, 1, false>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, slab); break;
        case kBinHeavy:
            num_heavy_kernel<<<heavy_grid(count, num_sms), kHeavyThreads, 0, st>>>(d_jobs, d_items, count, d_scratch,
                                                                                   max_ub, d_stats, d_err);
            break;
        default: break;
    }
}

}  // namespace spg
