// K4 numeric phase: row bins that run one row per CTA, the rows above 8192
// products (split into column-range pieces, or sorted in a global slab), and
// the bin dispatch (warp bins are compiled in k_numeric_warp.cu).  The per-row
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
                 int64_t cap, Stats* __restrict__ stats, ErrWord* __restrict__ err,
                 const unsigned long long* __restrict__ d_count) {
    if (d_count) count = static_cast<int64_t>(*d_count);  // rows left over by the piece planner
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

// ---------------------------------------------------------------------------
// Rows of more than kSplitThreshold products in upper-bound mode: split by
// column range into pieces of at most kPieceCap products, which run on the CTA
// pipeline of the 4096-product bin (8 warps x 16 products, values in a global
// slab, 3 CTAs per SM), many pieces of one row in parallel.  Those rows' own
// CTA kernels keep one 16-warp CTA per SM and leave most issue slots idle
// (25% of the warps resident); the pieces run at the occupancy of the CTA bins.
//
// split_plan_kernel, one CTA per row: enumerates the row once, stages every
// product (column, a*b) in product order in scratch and histograms the columns
// into kPlanBuckets buckets of the column space; then cuts greedily: each
// piece takes the longest run of buckets that still fits kPieceCap (a binary
// search over the bucket prefixes).  Rows with a bucket above kPieceCap or
// more than kMaxPieces pieces keep the global-slab path (num_heavy_kernel).  A
// piece owns the slots of its products in the row's reserved range (the
// products of earlier pieces have smaller columns, so they sort first).
// num_piece_kernel: each piece collects its range from the row's staging in
// product order (staged_products_in), then sorts, sums and writes like a row.
constexpr int kPlanThreads = 512;
constexpr int kPlanBuckets = 4096;
constexpr uint32_t kPieceCap = 4096;
constexpr int kMaxPieces = 256;
constexpr int kPieceW = 8, kPieceItems = 16, kPieceMinB = 3;
static_assert(kPieceW * 32 * kPieceItems >= static_cast<int>(kPieceCap), "a piece fits the CTA pipeline");

struct SplitPlan {
    unsigned long long* counters;  // [0] pieces, [1] rows left to the global-slab path, [2] staged products
    Piece* pieces;
    int64_t* fallback;
    int64_t max_pieces;
    int32_t* stage_col;  // staged products of the split rows (columns, values)
    double* stage_val;
    int64_t stage_cap;
};

struct PlanSmem {
    SegTab<kPlanThreads, int32_t> seg;
    int64_t warp_tmp[kPlanThreads / 32 + 1];
    uint32_t bucket[kPlanBuckets];  // counts, then exclusive prefixes
    int32_t start[kMaxPieces + 1];
    uint32_t maxc;
    int32_t npieces;
    unsigned long long base;
    unsigned long long stage;
};

__global__ void __launch_bounds__(kPlanThreads)
split_plan_kernel(const Job* __restrict__ jobs, const int64_t* __restrict__ items, int64_t count, SplitPlan plan,
                  ErrWord* __restrict__ err) {
    __shared__ PlanSmem sm;
    constexpr int kPer = kPlanBuckets / kPlanThreads;
    const int tid = threadIdx.x, lane = tid & 31;
    for (int64_t i = blockIdx.x; i < count; i += gridDim.x) {
        const int64_t it = items[i];
        const Job& J = jobs[item_job(it)];
        const int row = item_row(it);
        const int32_t ncols = J.B.cols;
        const int64_t P = J.ub[row];
        const int shift = max(0, ceil_log2(max(ncols, 1)) - 12);  // 4096 << shift >= ncols
        for (int k = tid; k < kPlanBuckets; k += kPlanThreads) sm.bucket[k] = 0;
        if (tid == 0) {
            sm.maxc = 0;
            sm.stage = atomicAdd(plan.counters + 2, static_cast<unsigned long long>(P));
        }
        __syncthreads();
        const bool staged = sm.stage + static_cast<unsigned long long>(P) <= static_cast<unsigned long long>(plan.stage_cap);
        if (!staged && tid == 0) raise_error(err, kErrOverflow, 9, row);
        int32_t* scol = plan.stage_col + (staged ? sm.stage : 0);
        double* sval = plan.stage_val + (staged ? sm.stage : 0);
        team_products<kPlanThreads, true, int32_t>(J, row, sm.seg, sm.warp_tmp, tid,
                                                   [&](int32_t seq, int32_t c, double b, double a) {
                                                       if (c < 0 || c >= ncols) {
                                                           raise_error(err, kErrInvalid, 4, c);
                                                           c = 0;
                                                       }
                                                       atomicAdd(&sm.bucket[c >> shift], 1u);
                                                       if (staged && seq < P) {
                                                           scol[seq] = c;
                                                           sval[seq] = __dmul_rn(a, b);
                                                       }
                                                   });
        uint32_t v[kPer];
        uint32_t sum = 0, mx = 0;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            v[j] = sm.bucket[tid * kPer + j];
            sum += v[j];
            mx = max(mx, v[j]);
        }
        mx = warp_max(mx);
        if (lane == 0) atomicMax(&sm.maxc, mx);
        uint32_t run = block_incl_scan<kPlanThreads>(sum, sm.warp_tmp) - sum;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            sm.bucket[tid * kPer + j] = run;
            run += v[j];
        }
        __syncthreads();
        const uint32_t total = static_cast<uint32_t>(P);
        if (tid == 0) {
            // greedy cut: prefix(e) = sm.bucket[e] (exclusive) for e < kPlanBuckets, total at the end
            auto prefix = [&](int e) { return e < kPlanBuckets ? sm.bucket[e] : total; };
            int np = 0, k = 0;
            bool ok = staged && sm.maxc <= kPieceCap;
            while (ok && k < kPlanBuckets) {
                if (np == kMaxPieces) {
                    ok = false;
                    break;
                }
                sm.start[np++] = k;
                int lo = k + 1, hi = kPlanBuckets;  // largest e in [lo, hi] with prefix(e) - prefix(k) <= cap
                const uint32_t limit = prefix(k) + kPieceCap;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (prefix(mid) <= limit) lo = mid;
                    else hi = mid - 1;
                }
                k = lo;
            }
            sm.npieces = ok ? np : 0;
            if (ok) {
                sm.start[np] = kPlanBuckets;
                sm.base = atomicAdd(plan.counters, static_cast<unsigned long long>(np));
                if (sm.base + np > static_cast<unsigned long long>(plan.max_pieces))
                    raise_error(err, kErrOverflow, 7, static_cast<int64_t>(sm.base + np));
            } else {
                plan.fallback[atomicAdd(plan.counters + 1, 1ull)] = it;
            }
        }
        __syncthreads();
        if (tid < sm.npieces && sm.base + tid < static_cast<unsigned long long>(plan.max_pieces)) {
            const int k0 = sm.start[tid], k1 = sm.start[tid + 1];
            Piece pc;
            pc.item = it;
            pc.lo = k0 << shift;
            pc.hi = k1 < kPlanBuckets ? (k1 << shift) : INT32_MAX;
            pc.slot_off = sm.bucket[k0];
            pc.count = static_cast<int64_t>(k1 < kPlanBuckets ? sm.bucket[k1] : total) - pc.slot_off;
            pc.scol = scol;
            pc.sval = sval;
            plan.pieces[sm.base + tid] = pc;
        }
        __syncthreads();
    }
}

template <int W, int ITEMS, int MINB>
__global__ void __launch_bounds__(W * 32, MINB)
num_piece_kernel(const Job* __restrict__ jobs, SplitPlan plan, Stats* __restrict__ stats, ErrWord* __restrict__ err,
                 double* __restrict__ gvals, unsigned long long* __restrict__ ticket) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ RowQueue q;  // pieces from the launch's queue, as the row kernels take rows
    using Sm = RowSmem<W, ITEMS, false>;
    Sm& sm = *reinterpret_cast<Sm*>(smem_raw);
    double* vals = gvals + static_cast<size_t>(blockIdx.x) * Sm::kCap;
    const int64_t count = min(static_cast<int64_t>(*plan.counters), plan.max_pieces);
    unsigned long long mine = 0;
    int par = 0;
    for (int64_t i = blockIdx.x; i < count; par ^= 1) {
        if (threadIdx.x == 0)
            q.next[par] = static_cast<int64_t>(gridDim.x) + static_cast<int64_t>(atomicAdd(ticket, 1ull));
        const Piece pc = plan.pieces[i];
        if (pc.count > 0) {
            const Job& J = jobs[item_job(pc.item)];
            mine += numeric_row<W, ITEMS, false, true>(J, item_row(pc.item), sm, vals, err, &pc);
        } else {
            __syncthreads();  // an empty last piece (same for the whole CTA): no row barrier orders the queue
        }
        i = q.next[par];
    }
    if (mine) atomicAdd(&stats->nz_total, mine);
}

// Scratch layout of the split rows (upper-bound mode): counters | pieces |
// fallback rows | staged columns | staged values | slabs (the pieces' value
// slabs, then the global-slab sort of the fallback rows: one after the other).
struct SplitLayout {
    size_t pieces_off, fallback_off, col_off, val_off, slab_off, bytes;
    int64_t max_pieces;
};

int heavy_grid(int64_t count, int num_sms);

// Depends only on the call's totals, so that the launches of bins 17-19 (one
// after the other on one stream) lay the same scratch out identically.
SplitLayout split_layout(int64_t max_ub, const SplitTotals& split, int num_sms) {
    SplitLayout L;
    const int64_t rows = split.rows, split_products = split.products;
    // two neighbouring greedy pieces of a row together exceed the cap: at most
    // 2 * ub / cap + 1 pieces per row
    L.max_pieces = 2 * split_products / kPieceCap + rows;
    auto up = [](size_t x) { return (x + 255) & ~size_t{255}; };
    L.pieces_off = 256;
    L.fallback_off = up(L.pieces_off + static_cast<size_t>(L.max_pieces) * sizeof(Piece));
    L.col_off = up(L.fallback_off + static_cast<size_t>(rows) * sizeof(int64_t));
    L.val_off = up(L.col_off + static_cast<size_t>(split_products) * sizeof(int32_t));
    L.slab_off = up(L.val_off + static_cast<size_t>(split_products) * sizeof(double));
    const size_t piece_slab = static_cast<size_t>(num_sms) * kPieceMinB * kPieceW * 32 * kPieceItems * sizeof(double);
    const size_t global_slab = static_cast<size_t>(heavy_grid(rows, num_sms)) * 24 * static_cast<size_t>(max_ub);
    L.bytes = L.slab_off + std::max(piece_slab, global_slab);
    return L;
}

int heavy_grid(int64_t count, int num_sms) { return static_cast<int>(count < num_sms ? count : num_sms); }

// Product-value slab of one CTA of the two global-slab bins.
constexpr int64_t slab_cap(int bin) { return bin == 17 ? 16 * 32 * 24 : 16 * 32 * 32; }

// Team shapes of the bins of 769-1536 and 2049-8192 products: warps, products
// per thread, CTAs per SM, product values in shared memory (else in a per-CTA
// global slab at the end of the scratch).  With the values in slabs, shared
// memory stops limiting the resident CTAs, and more CTAs per SM hide each
// other's barriers.  Measured on the power-law workload, one bin at a time:
//   1024: 2x16, 8 CTAs/SM, shared values    1.48 ms -> 2x16, 12 CTAs/SM, slab 1.34 ms
//         (9 CTAs/SM with shared values 1.56 ms, 10 with a slab 1.46 ms)
//   1536: 8x6, 4 CTAs/SM, shared values     1.99 ms -> 4x12, 8 CTAs/SM, slab 1.90 ms
//         (8x6 at 5 CTAs/SM with a slab 2.02 ms)
//   3072: 12x8, 2 CTAs/SM, shared values    1.99 ms -> 8x12, 4 CTAs/SM, slab 1.67 ms
//   4096: 8x16, 2 CTAs/SM, shared values    1.12 ms -> 8x16, 3 CTAs/SM, slab 1.00 ms
//         (8x16 at 4 CTAs/SM with a slab 0.97 ms, 16x8 at 2 1.02 ms)
//   6144: 16x12, 1 CTA/SM, shared values    1.55 ms -> 16x12, 2 CTAs/SM, slab 1.34 ms
//         (8x24 at 3 CTAs/SM 1.42 ms, 12x16 at 2 1.33 ms against 1.28)
//   8192: 16x16, 1 CTA/SM, shared values    0.73 ms (2 CTAs/SM with a slab: the same)
// The slabs of these bins share one region: the bins run one after the other
// on one stream.
constexpr int kB10W = 2, kB10I = 16, kB10MinB = 12;
constexpr bool kB10SV = false;
constexpr int kB11W = 4, kB11I = 12, kB11MinB = 8;
constexpr bool kB11SV = false;
constexpr int kB13W = 8, kB13I = 12, kB13MinB = 4;
constexpr bool kB13SV = false;
constexpr int kB14W = 8, kB14I = 16, kB14MinB = 3;
constexpr bool kB14SV = false;
constexpr int kB15W = 16, kB15I = 12, kB15MinB = 2;
constexpr bool kB15SV = false;
constexpr int kB16W = 16, kB16I = 16, kB16MinB = 1;
constexpr bool kB16SV = true;

// Bytes of the value slabs of bins 10, 11 and 13-16 (0 for a bin whose values
// are in shared memory).
size_t cta_slab_bytes(int bin, int64_t count, int num_sms) {
    auto f = [&](int w, int items, int minb, bool sv) -> size_t {
        if (sv || count <= 0) return 0;
        const int64_t grid = std::min<int64_t>(count, static_cast<int64_t>(num_sms) * minb);
        return static_cast<size_t>(grid) * w * 32 * items * sizeof(double);
    };
    switch (bin) {
        case 10: return f(kB10W, kB10I, kB10MinB, kB10SV);
        case 11: return f(kB11W, kB11I, kB11MinB, kB11SV);
        case 13: return f(kB13W, kB13I, kB13MinB, kB13SV);
        case 14: return f(kB14W, kB14I, kB14MinB, kB14SV);
        case 15: return f(kB15W, kB15I, kB15MinB, kB15SV);
        case 16: return f(kB16W, kB16I, kB16MinB, kB16SV);
        default: return 0;
    }
}

}  // namespace

size_t numeric_scratch_bytes(const int64_t* bin_count, int64_t max_ub, const SplitTotals& split, int num_sms,
                             bool holes, bool concurrent) {
    // Bins 17-19 share the front of the scratch (they run one after the other);
    // bins 10, 11 and 13-16 take their slabs from its end (also one after the
    // other), after that region when the two groups run on concurrent streams.
    size_t cta = 0;
    for (int b = 10; b <= 16; ++b) cta = std::max(cta, cta_slab_bytes(b, bin_count[b], num_sms));
    size_t need = 0;
    if (holes) {
        if (split.rows > 0) need = split_layout(max_ub, split, num_sms).bytes;
        // bins 17 and 18 run whole where the autotuner chose it (same region:
        // these launches run one after the other on one stream)
        for (int b = kLastSmemBin + 1; b < kBinHeavy; ++b)
            if (bin_count[b])
                need = std::max(need, static_cast<size_t>(slab_grid(bin_count[b], num_sms)) * slab_cap(b) * sizeof(double));
    } else {
        for (int b = kLastSmemBin + 1; b < kBinHeavy; ++b)  // the launches run one after the other
            if (bin_count[b])
                need = std::max(need, static_cast<size_t>(slab_grid(bin_count[b], num_sms)) * slab_cap(b) * sizeof(double));
        const int64_t heavy = bin_count[kBinHeavy];
        if (heavy)
            need = std::max(need, static_cast<size_t>(heavy_grid(heavy, num_sms)) * 24 * static_cast<size_t>(max_ub));
    }
    return concurrent ? ((need + 255) & ~size_t{255}) + cta : std::max(need, cta);
}

// The last `need` bytes of the scratch (nullptr when none are needed).
static double* tail_slab(void* d_scratch, size_t scratch_bytes, size_t need) {
    return need ? reinterpret_cast<double*>(static_cast<unsigned char*>(d_scratch) + (scratch_bytes - need)) : nullptr;
}

// Rows of more than kSplitThreshold products in upper-bound mode: plan and
// stage, the pieces, then the rows left to the global-slab sort.
static void launch_split(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, int64_t max_ub,
                         const SplitTotals& split, void* d_scratch, Stats* d_stats, ErrWord* d_err, cudaStream_t st,
                         int num_sms) {
    const SplitLayout L = split_layout(max_ub, split, num_sms);
    unsigned char* base = static_cast<unsigned char*>(d_scratch);
    SplitPlan plan;
    plan.counters = reinterpret_cast<unsigned long long*>(base);
    plan.pieces = reinterpret_cast<Piece*>(base + L.pieces_off);
    plan.fallback = reinterpret_cast<int64_t*>(base + L.fallback_off);
    plan.max_pieces = L.max_pieces;
    plan.stage_col = reinterpret_cast<int32_t*>(base + L.col_off);
    plan.stage_val = reinterpret_cast<double*>(base + L.val_off);
    plan.stage_cap = split.products;
    void* slabs = base + L.slab_off;
    cudaMemsetAsync(plan.counters, 0, 4 * sizeof(unsigned long long), st);
    split_plan_kernel<<<static_cast<int>(std::min<int64_t>(count, 3 * num_sms)), kPlanThreads, 0, st>>>(
        d_jobs, d_items, count, plan, d_err);
    using PieceSm = RowSmem<kPieceW, kPieceItems, false>;
    const int smem = static_cast<int>(sizeof(PieceSm));
    auto kern = num_piece_kernel<kPieceW, kPieceItems, kPieceMinB>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    // the bin's own queue: bins 17-19 each plan and run their pieces, one after the other
    kern<<<num_sms * kPieceMinB, kPieceW * 32, smem, st>>>(d_jobs, plan, d_stats, d_err, static_cast<double*>(slabs),
                                                          &d_stats->ticket[bin]);
    num_heavy_kernel<<<heavy_grid(count, num_sms), kHeavyThreads, 0, st>>>(
        d_jobs, plan.fallback, count, slabs, max_ub, d_stats, d_err, plan.counters + 1);
}

void launch_numeric(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, int64_t max_ub,
                    const SplitTotals& split, void* d_scratch, size_t scratch_bytes, Stats* d_stats, ErrWord* d_err,
                    cudaStream_t st, int num_sms, bool holes, int variant) {
    if (count <= 0) return;
    if (variant == 1 && launch_numeric_alt(bin, d_jobs, d_items, count, d_stats, d_err, st, num_sms)) return;
    if (bin <= kLastWarpBin) {
        launch_numeric_warp(bin, d_jobs, d_items, count, d_stats, d_err, st, num_sms);
        return;
    }
    // Rows above 8,192 products are split into column-range pieces in the
    // upper-bound layout; the alternative of bins 17 and 18 (8,193-16,384
    // products) runs those rows whole, one 16-warp CTA each, as the exact layout
    // does -- the autotuner keeps it where it measures faster.
    const bool whole = variant == 1 && bin < kBinHeavy;
    if (holes && bin > kLastSmemBin && !whole) {
        launch_split(bin, d_jobs, d_items, count, max_ub, split, d_scratch, d_stats, d_err, st, num_sms);
        return;
    }
    double* slab = static_cast<double*>(d_scratch);
    unsigned long long* const tk = &d_stats->ticket[bin];  // the bin's row queue
    switch (bin) {
        case 9: run_block<4, 6, 8>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); break;     // <= 768
        case 10:  // <= 1024
            run_block<kB10W, kB10I, kB10MinB, kB10SV>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk,
                                                     tail_slab(d_scratch, scratch_bytes, cta_slab_bytes(10, count, num_sms)));
            break;
        case 11:  // <= 1536
            run_block<kB11W, kB11I, kB11MinB, kB11SV>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk,
                                                     tail_slab(d_scratch, scratch_bytes, cta_slab_bytes(11, count, num_sms)));
            break;
        case 12: run_block<8, 8, 4>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); break;    // <= 2048
        case 13:  // <= 3072
            run_block<kB13W, kB13I, kB13MinB, kB13SV>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk,
                                                     tail_slab(d_scratch, scratch_bytes, cta_slab_bytes(13, count, num_sms)));
            break;
        case 14:  // <= 4096
            run_block<kB14W, kB14I, kB14MinB, kB14SV>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk,
                                                     tail_slab(d_scratch, scratch_bytes, cta_slab_bytes(14, count, num_sms)));
            break;
        case 15:  // <= 6144
            run_block<kB15W, kB15I, kB15MinB, kB15SV>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk,
                                                     tail_slab(d_scratch, scratch_bytes, cta_slab_bytes(15, count, num_sms)));
            break;
        case 16:  // <= 8192
            run_block<kB16W, kB16I, kB16MinB, kB16SV>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk,
                                                     tail_slab(d_scratch, scratch_bytes, cta_slab_bytes(16, count, num_sms)));
            break;
        case 17: run_block<16, 24, 1, false>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk, slab); break;
        case 18: run_block<16, 32, 1, false>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk, slab); break;
        case kBinHeavy:  // exact layout (the upper-bound layout splits these rows)
            num_heavy_kernel<<<heavy_grid(count, num_sms), kHeavyThreads, 0, st>>>(
                d_jobs, d_items, count, d_scratch, max_ub, d_stats, d_err, nullptr);
            break;
        default: break;
    }
}

}  // namespace spg
