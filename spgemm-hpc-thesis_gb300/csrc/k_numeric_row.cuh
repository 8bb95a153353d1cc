// K4 numeric phase: every output row sorted, summed and written without zeros.
//
// For a row with P products the kernel
//   1. enumerates the products in reference order (spg_enum.cuh): product t gets
//      its column, sequence number t and value __dmul_rn(a, b) (one rounding, as
//      `const double product = aValue * b` in spgemm_exchange.cpp:287);
//   2. sorts the products by column with a stable LSD radix sort (8-bit digits
//      over the bits of max(col) - min(col) only; ranks from ballot-matched
//      lane groups and per-warp digit counters), so that equal columns stay in
//      product order.
//      When the column range and the sequence number fit in 32 bits together,
//      the sort moves one packed word (column - min) << s | seq per product;
//      otherwise it moves the column and a 16-bit sequence number side by side;
//   3. sums each run of equal columns sequentially in product order with
//      __dadd_rn, starting from its first product (the `emplace` then `+=` of
//      spgemm_exchange.cpp:288-293), and keeps the sums that are != 0.0
//      (spgemm_exchange.cpp:304; NaN and infinities are kept);
//   4. writes the kept (column, sum) pairs, already in column order, at the
//      row's output offset (job.cnt[row]) and the kept count into job.nz[row].
// Every coordinate is therefore bit-identical to the serial reference.  Rows of
// <= 512 products run one per warp (num_warp_kernel), rows of <= 8192 one per
// CTA with the keys in shared memory and the values in shared memory or a
// per-CTA global slab (num_block_kernel).  Heavier rows are split by column
// range into pieces that run on the same pipeline (num_piece_kernel) in the
// upper-bound layout; in the exact layout rows of <= 16384 run one per CTA with
// a value slab and heavier ones with the whole sort in a global slab
// (num_heavy_kernel, k_numeric.cu).
#pragma once

#include <atomic>

#include <type_traits>

#include "spg_enum.cuh"

namespace spg {
namespace {

template <int W>
__device__ inline void row_sync() {
    if (W == 1) __syncwarp();
    else __syncthreads();
}

constexpr int log2_ceil_c(int x) { return x <= 1 ? 0 : 1 + log2_ceil_c((x + 1) / 2); }

// Digit counters of W warps: counter (digit d, warp w) lives at hidx<W>(d, w),
// digit-major with an odd stride kHistStride >= W, so that the counters one
// warp's lanes touch for different digits fall in different banks (with stride
// W they would share 32 / W banks).
template <int W>
constexpr int kHistStride = W == 1 ? 1 : (W % 2 == 0 ? W + 1 : W + 2);
template <int W>
constexpr int kHistWords = 256 * kHistStride<W>;
template <int W>
__device__ __forceinline__ int hidx(int d, int w) {
    return W == 1 ? d : d * kHistStride<W> + w;
}

// Bucket sort (bucket_sort below): 2^kCoarseBits<W> coarse buckets (256 for a
// CTA row, 32 for a warp row), whose 16-bit counters take kBkCoarseWords<W>
// words and whose table (first fine bucket, fine bits) kBkInfoWords<W>; then
// the fine counters.  (7 coarse bits for CTA rows measured 0.25 ms slower on
// the power-law product.)
template <int W>
constexpr int kCoarseBits = W == 1 ? 5 : 8;
template <int W>
constexpr int kBkCoarseWords = (1 << kCoarseBits<W>) / 2;
template <int W>
constexpr int kBkInfoWords = 1 << kCoarseBits<W>;
// Fine bits of a coarse bucket of n products: floor(log2 n) + fine_extra(cap)
// (at most the bucket's column bits), so P products take at most
// P << fine_extra(cap) fine counters, plus one past the last; fine bucket
// numbers stay below 2^16 (they are stored in 16-bit words).  On the power-law
// product one extra bit for CTA rows measured 1.1% faster than none (buckets
// of 0.5-1 products on average instead of 1-2: shorter rank loops), two 5%
// slower; for warp rows one extra bit measured 4% slower than none.
constexpr int kFineExtraBits = 1;
constexpr int kWarpFineExtraBits = 0;
constexpr int fine_extra(int cap, int w = 2) {
    int e = w == 1 ? kWarpFineExtraBits : kFineExtraBits;
    while (e > 0 && (cap << e) >= 65536) --e;
    return e;
}
template <int W, int ITEMS>
constexpr int kBkWords = kBkCoarseWords<W> + kBkInfoWords<W> + ((W * 32 * ITEMS) << fine_extra(W * 32 * ITEMS, W)) / 2 + 1;

// In the packed layout the scatter also stores every product's fine bucket
// beside it (in the sequence-number array, which that layout leaves unused),
// so that ranking a position reads its bucket instead of recomputing it from
// the coarse table (0.29 ms of K4 on the power-law product).
constexpr bool kStoreFine = true;
// The fine histogram keeps every product's arrival index in its bucket (the
// counter's old value), so the scatter places products at bucket start plus
// arrival with no second round of atomics.
constexpr bool kArrivalScatter = true;
// Products ranked together in the bucket sort's rank step (see bucket_sort):
// the largest divisor of ITEMS not above kRankGroup.  On the power-law product:
// one at a time 13.96 ms of K4, two 13.75, four 13.91, six 13.87 (register
// pressure grows with the group).
constexpr int kRankGroup = 2;
constexpr int rank_group(int items) {
    for (int g = kRankGroup; g > 1; --g)
        if (items % g == 0) return g;
    return 1;
}
// Which rows take the bucket sort: CTA rows, and warp rows of 8-16 products per
// lane (32 coarse buckets, no extra fine bit, so that a warp's counters stay
// small).  On the power-law product, with the bins on three streams, K4 took
// 12.64 -> 12.10 ms, uniform 0.204 -> 0.199 ms; on one stream the 512-product
// bin alone is slower (0.77 -> 0.94 ms: a warp row's passes need no barrier,
// so the radix sort's extra instructions cost little while the bin runs
// alone), but beside the CTA bins the fewer instructions win.  Warp rows of 6
// products per lane measured the same either way; fewer keep the radix sort.
constexpr int kWarpBucketMinItems = 8;
constexpr int kWarpBucketMaxItems = 16;
template <int W, int ITEMS>
constexpr bool kBucketRows = W > 1 || (ITEMS >= kWarpBucketMinItems && ITEMS <= kWarpBucketMaxItems);
// A fine bucket holding more products than this (a column repeated many times)
// sends the row to the radix sort: ranking inside a bucket is quadratic.
constexpr uint32_t kMaxFine = 64;

// Digit-counter sets of CTA rows.  CTA rows take the radix sort only where the
// bucket sort declines, so one set (an extra barrier per pass) leaves them more
// shared memory.
constexpr int kHistSets = 1;

// SV: product values in shared memory (else in a per-CTA global slab).
template <int W, int ITEMS, bool SV = true>
struct RowSmem {
    static constexpr int kCap = W * 32 * ITEMS;
    static constexpr int kSeqBits = log2_ceil_c(kCap);
    double vals[SV ? kCap : 1];  // product values by sequence number; run sums in place
    RowSegs<W * 32, W * 32 * ITEMS> seg;  // enumeration batch
    int64_t warp_tmp[W + 1];    // block scans
    uint32_t keys[kCap];        // columns (unpacked) or packed (column, sequence) words
    union {
        // digit counters of the radix sort at hidx<W>(digit, warp); with two
        // sets (kHistSets) CTA rows alternate them so that clearing the next
        // pass's set needs no barrier of its own
        alignas(16) uint32_t hist[W == 1 ? 1 : kHistSets][kHistWords<W>];
        // bucket sort of CTA rows: coarse counters, coarse bucket table, fine
        // counters (16-bit counters, two per word)
        alignas(16) uint32_t bk[kBucketRows<W, ITEMS> ? kBkWords<W, ITEMS> : 1];
    };
    uint32_t cnt[W * ITEMS];    // kept entries per (warp, item)
    uint16_t seqs[kCap];        // sequence numbers of the unpacked path
    int32_t red[2 * W];         // min / max column reduction
    uint32_t step_cnt[64];      // kept counts of one filtered enumeration step (row pieces)
};

// Exclusive scan of the NDIG*W digit counters in (digit, warp) order (logical
// index L = d * W + w): NDIG/32 consecutive counters per thread, one for the
// first 16*W threads when NDIG is 16.
template <int W, int NDIG = 256>
__device__ inline void scan_counters(uint32_t* c, int64_t* tmp) {
    constexpr int kPer = NDIG >= 32 ? NDIG / 32 : 1;
    constexpr int kTot = NDIG * W;
    const int lane = threadIdx.x & 31;
    const int warp = W == 1 ? 0 : (threadIdx.x >> 5);
    const int tid = W == 1 ? lane : threadIdx.x;
    const bool act = NDIG >= 32 || tid < kTot;
    auto phys = [](int L) { return W == 1 ? L : hidx<W>(L / W, L % W); };
    uint32_t v[kPer];
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        v[j] = act ? c[phys(tid * kPer + j)] : 0u;
        sum += v[j];
    }
    const uint32_t incl = warp_incl_scan(sum, lane);
    uint32_t base = incl - sum;
    if (W > 1) {  // every warp scans the W warp totals itself: one barrier
        if (lane == 31) tmp[warp] = incl;
        __syncthreads();
        const uint32_t t = lane < W ? static_cast<uint32_t>(tmp[lane]) : 0u;
        base += __shfl_sync(0xffffffffu, warp_incl_scan(t, lane) - t, warp);
    }
    if (act) {
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            c[phys(tid * kPer + j)] = base;
            base += v[j];
        }
    }
}

// Zeroes the counters of the first ndig digits (ndig * kHistStride<W> words, a
// multiple of four) with 16-byte stores; h is 16-byte aligned.
template <int W>
__device__ inline void clear_counters(uint32_t* h, int ndig, int tid) {
    uint4* h4 = reinterpret_cast<uint4*>(h);
    const int n4 = ndig * kHistStride<W> / 4;
    for (int d = tid; d < n4; d += W * 32) h4[d] = make_uint4(0u, 0u, 0u, 0u);
}

// Lanes of the warp holding the same NB-bit digit: the intersection of one
// ballot per digit bit (a ballot for each set bit, its complement for each
// clear bit).  Eight votes cost a fraction of one __match_any_sync on GB300.
template <int NB = 8>
__device__ inline unsigned digit_peers(uint32_t d) {
    unsigned peers = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const unsigned bit = (d >> b) & 1u;
        const unsigned set = __ballot_sync(0xffffffffu, bit);
        peers &= set ^ (bit - 1u);  // set where this lane's bit is 1, ~set where it is 0
    }
    return peers;
}

// Stable rank of one striped item against this warp's digit counters: the
// group of lanes holding the same digit (digit_peers); its first lane advances
// the counter by the group size (one shared atomic) and broadcasts the old
// value.  Items of a warp are ranked in order, so ranks follow
// (warp, item, lane) order.
template <int NB = 8>
__device__ inline uint32_t rank_item(uint32_t d, uint32_t* counter_of_d, int lane) {
    const unsigned peers = digit_peers<NB>(d);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter_of_d, static_cast<uint32_t>(__popc(peers)));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(peers & lanemask_lt());
}

// Exclusive scan of the W*ITEMS per-(warp, item) kept counts by warp 0; the
// total goes to red[0].
template <int W, int ITEMS>
__device__ inline void scan_kept(uint32_t* cnt, int32_t* red, int warp, int lane) {
    constexpr int kN = W * ITEMS;
    constexpr int kPer = (kN + 31) / 32;
    if (warp == 0) {
        uint32_t v[kPer];
        uint32_t tot = 0;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const int idx = lane * kPer + j;
            v[j] = idx < kN ? cnt[idx] : 0u;
            tot += v[j];
        }
        const uint32_t incl = warp_incl_scan(tot, lane);
        uint32_t base = incl - tot;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const int idx = lane * kPer + j;
            if (idx < kN) cnt[idx] = base;
            base += v[j];
        }
        if (lane == 31) red[0] = static_cast<int32_t>(incl);
    }
}

// Where a row's result goes, read once from the Job (locals, not reloaded
// through the Job reference after every global store).
struct RowOut {
    int32_t* __restrict__ c_col;
    double* __restrict__ c_val;
    int64_t out0;       // first slot of the row in C_tmp
    int64_t* nz;        // the row's stored-entry count
    int32_t holes;      // upper-bound mode: slot-per-position output with holes
    int32_t nz_add;     // a piece of a split row: add to *nz instead of storing it
};

// 16-bit counter i of an array of packed pairs (low half: even i).
__device__ __forceinline__ uint32_t half16(const uint32_t* a, uint32_t i) {
    return (a[i >> 1] >> ((i & 1u) << 4)) & 0xffffu;
}
// Adds one to 16-bit counter i and returns its previous value.
__device__ __forceinline__ uint32_t bump16(uint32_t* a, uint32_t i) {
    const uint32_t sh = (i & 1u) << 4;
    return (atomicAdd(&a[i >> 1], 1u << sh) >> sh) & 0xffffu;
}
// bump16 for every valid lane of a warp (all 32 lanes call it), one atomic per
// run of consecutive lanes with the same counter: consecutive products of one
// B row mostly fall into the same coarse bucket, and a shared atomic that many
// lanes aim at one word is serialised.  Valid lanes are a prefix of the warp.
__device__ __forceinline__ void bump16_runs(uint32_t* a, uint32_t i, bool valid, int lane) {
    const uint32_t prev = __shfl_up_sync(0xffffffffu, i, 1);
    const bool head = valid && (lane == 0 || prev != i);
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    if (head) {
        const unsigned later = heads & ~((2u << lane) - 1u);  // heads after this lane (lane 31: none)
        const int next = later ? __ffs(later) - 1 : __popc(vmask);
        atomicAdd(&a[i >> 1], static_cast<uint32_t>(next - lane) << ((i & 1u) << 4));
    }
}

// Exclusive scan of v over the W*32 threads of a row's team in thread order,
// with the total and the team-wide maximum of m (red: 2*W words; one barrier
// for a CTA, none for a warp).  red is next written after later barriers of
// the row, so no barrier protects it here.
template <int W>
__device__ inline uint32_t block_excl_scan_max(uint32_t v, uint32_t m, int32_t* red, int lane, int warp,
                                               uint32_t& total, uint32_t& mx) {
    const uint32_t incl = warp_incl_scan(v, lane);
    const uint32_t wm = __reduce_max_sync(0xffffffffu, m);
    if constexpr (W == 1) {
        total = __shfl_sync(0xffffffffu, incl, 31);
        mx = wm;
        return incl - v;
    }
    if (lane == 31) {
        red[warp] = static_cast<int32_t>(incl);
        red[W + warp] = static_cast<int32_t>(wm);
    }
    __syncthreads();
    uint32_t base = 0, tot = 0, gm = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const uint32_t s = static_cast<uint32_t>(red[w]);
        base += w < warp ? s : 0u;
        tot += s;
        gm = max(gm, static_cast<uint32_t>(red[W + w]));
    }
    total = tot;
    mx = gm;
    return base + incl - v;
}

// Zeroes the bucket sort's coarse counters and the fine counters of a row of P
// products, which the sort expects to find cleared.  Called before the row's
// enumeration, whose barriers order it before the sort's first atomics; the
// previous row's sort ended with barriers, so no warp still reads them.
template <int W, int ITEMS, bool SV>
__device__ __forceinline__ void clear_buckets(RowSmem<W, ITEMS, SV>& sm, int P, int tid) {
    constexpr int kExtra = fine_extra(RowSmem<W, ITEMS, SV>::kCap, W);
    static_assert((RowSmem<W, ITEMS, SV>::kCap << kExtra) < 65536, "fine bucket numbers are 16-bit");
    uint32_t* fc = sm.bk + kBkCoarseWords<W> + kBkInfoWords<W>;
    const int fwords = ((P << kExtra) + 2) >> 1;
    for (int i = tid; i < kBkCoarseWords<W>; i += W * 32) sm.bk[i] = 0u;
    for (int i = tid; i < fwords; i += W * 32) fc[i] = 0u;
}

// Step 2 of a CTA row without digit passes: the products (columns at
// keys[0..P), offsets k = column - cmin of nbits >= 1 bits, sequence number =
// position) are bucketed, then ranked inside their bucket.
//   * coarse buckets: the top min(nbits, 8) bits of k (16-bit counters);
//   * coarse bucket c of n_c products gets 2^fb_c fine buckets over its column
//     span, fb_c = min(span bits, floor(log2 n_c)), so that dense parts of the
//     row (the diagonal band of a banded product) get finer buckets than sparse
//     ones and no more fine buckets than products exist;
//   * the products are scattered into their fine buckets in any order (shared
//     atomics), then every product finds its place in its bucket by counting
//     the bucket's products with a smaller (column, sequence) pair: the pair is
//     unique, so the result is the order of a stable sort by column, the
//     reference's order of every column's products.
// Instruction cost per product does not grow with the column range, unlike a
// digit pass.  Returns false, leaving keys untouched, when a fine bucket would
// hold more than kMaxFine products (a column repeated that often); the row then
// takes the radix sort.  On success keys (and seqs when !PACKED) hold the sorted
// products in the layout finish_row reads: packed (column - cmin, sequence)
// words, or columns and 16-bit sequence numbers side by side.
template <int W, int ITEMS, bool SV, bool PACKED>
__device__ bool bucket_sort(RowSmem<W, ITEMS, SV>& sm, int P, uint32_t cmin, int nbits, int lane, int warp,
                            int tid) {
    using Sm = RowSmem<W, ITEMS, SV>;
    constexpr int NT = W * 32;
    constexpr int kSeqBits = Sm::kSeqBits;
    static_assert(kBucketRows<W, ITEMS>, "rows of this shape have no bucket counters");
    uint32_t* cc = sm.bk;                                     // coarse counters
    uint32_t* info = sm.bk + kBkCoarseWords<W>;                  // first fine bucket | fine bits << 16
    uint32_t* fc = sm.bk + kBkCoarseWords<W> + kBkInfoWords<W>;     // fine counters, then starts, then ends
    const int cbits = nbits < kCoarseBits<W> ? nbits : kCoarseBits<W>;
    const int sc = nbits - cbits;                             // column bits inside a coarse bucket
    const uint32_t scmask = (1u << sc) - 1u;
    // 0. the coarse counters and the fine counters of P products are zero on
    //    entry (clear_buckets, before the row's enumeration)
    constexpr int kExtra = fine_extra(Sm::kCap, W);
    const int fwords = ((P << kExtra) + 2) >> 1;  // one counter past the last fine bucket
    // 1. coarse histogram
    uint32_t k[ITEMS], f[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const int pos = (warp * ITEMS + i) * 32 + lane;
        k[i] = pos < P ? sm.keys[pos] - cmin : 0u;
        bump16_runs(cc, k[i] >> sc, pos < P, lane);
    }
    row_sync<W>();
    // 2. fine buckets of every coarse bucket, numbered in coarse order: every
    //    warp computes the whole table and stores it (the same words with the
    //    same values), so that only a warp-level barrier precedes its use
    {
        constexpr int kPer = (1 << kCoarseBits<W>) / 32;  // coarse buckets per lane
        uint32_t fcount[kPer], fbits[kPer], sum = 0;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t n = half16(cc, static_cast<uint32_t>(lane * kPer + j));  // zero beyond 2^cbits
            const int lg = n ? 31 - __clz(n) + kExtra : 0;
            fbits[j] = static_cast<uint32_t>(lg < sc ? lg : sc);
            fcount[j] = n ? (1u << fbits[j]) : 0u;
            sum += fcount[j];
        }
        uint32_t base = warp_incl_scan(sum, lane) - sum;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            info[lane * kPer + j] = base | (fbits[j] << 16);
            base += fcount[j];
        }
    }
    __syncwarp();
    // 3. fine histogram
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const int pos = (warp * ITEMS + i) * 32 + lane;
        f[i] = 0u;
        if (pos < P) {
            const uint32_t in = info[k[i] >> sc];
            f[i] = (in & 0xffffu) + ((k[i] & scmask) >> (sc - static_cast<int>(in >> 16)));
            if constexpr (kArrivalScatter) f[i] |= bump16(fc, f[i]) << 16;  // arrival in the high half
            else bump16(fc, f[i]);
        }
    }
    row_sync<W>();
    // 4. exclusive scan of the fine counters (at most P of them; contiguous
    //    words per thread), and the largest fine bucket
    {
        const int per = (fwords + NT - 1) / NT;
        const int w0 = tid * per;
        const int w1 = min(w0 + per, fwords);
        uint32_t sum = 0, mx = 0;
        for (int w = w0; w < w1; ++w) {
            const uint32_t x = fc[w];
            const uint32_t lo = x & 0xffffu, hi = x >> 16;
            sum += lo + hi;
            mx = max(mx, max(lo, hi));
        }
        uint32_t total, gmax;
        uint32_t base = block_excl_scan_max<W>(sum, mx, sm.red, lane, warp, total, gmax);
        if (gmax > kMaxFine) return false;  // uniform: every thread saw the same maximum
        for (int w = w0; w < w1; ++w) {
            const uint32_t x = fc[w];
            const uint32_t lo = x & 0xffffu;
            fc[w] = base | ((base + lo) << 16);
            base += lo + (x >> 16);
        }
    }
    row_sync<W>();
    // 5. scatter into the fine buckets (any order inside a bucket)
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const int pos = (warp * ITEMS + i) * 32 + lane;
        if (pos < P) {
            const uint32_t fi = f[i] & 0xffffu;
            const uint32_t at = kArrivalScatter ? half16(fc, fi) + (f[i] >> 16) : bump16(fc, fi);
            if constexpr (PACKED) {
                sm.keys[at] = (k[i] << kSeqBits) | static_cast<uint32_t>(pos);
                if constexpr (kStoreFine) sm.seqs[at] = static_cast<uint16_t>(fi);
            } else {
                sm.keys[at] = k[i] + cmin;  // the unpacked layout keeps columns
                sm.seqs[at] = static_cast<uint16_t>(pos);
            }
        }
    }
    row_sync<W>();
    // 6. every sorted position takes its product's place inside the product's
    //    bucket: the number of the bucket's products with a smaller (column,
    //    sequence) pair.  Positions run in lane order, so the lanes of a warp
    //    mostly share buckets (same loop bounds, broadcast loads).  The counters
    //    hold every bucket's start (arrival scatter; the one past the last bucket
    //    holds P) or its end.
    uint32_t* const dst = f;  // the fine indices are no longer needed
    uint32_t* const key = k;  // nor the column offsets
    uint32_t sqv[PACKED ? 1 : ITEMS];  // sequence numbers of the unpacked layout
    // Positions are ranked kRankGroup at a time in lock-step: their buckets'
    // bounds are loaded together, then one loop over the longest of their
    // buckets issues independent loads for all of them.
    constexpr int G = rank_group(ITEMS);
#pragma unroll
    for (int i0 = 0; i0 < ITEMS; i0 += G) {
        uint32_t beg[G], len[G], r[G], maxlen = 0;
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int i = i0 + g;
            const int p = (warp * ITEMS + i) * 32 + lane;
            key[i] = 0u;
            beg[g] = 0u;
            len[g] = 0u;
            r[g] = 0u;
            if (p < P) {
                key[i] = sm.keys[p];
                uint32_t fb;
                if constexpr (PACKED && kStoreFine) {
                    fb = sm.seqs[p];
                } else {
                    const uint32_t kk = PACKED ? key[i] >> kSeqBits : key[i] - cmin;
                    const uint32_t in = info[kk >> sc];
                    fb = (in & 0xffffu) + ((kk & scmask) >> (sc - static_cast<int>(in >> 16)));
                }
                if constexpr (!PACKED) sqv[i] = sm.seqs[p];
                // counters hold bucket starts (arrival scatter) or ends
                const uint32_t end = kArrivalScatter ? half16(fc, fb + 1u) : half16(fc, fb);
                beg[g] = kArrivalScatter ? half16(fc, fb) : (fb ? half16(fc, fb - 1u) : 0u);
                len[g] = end - beg[g];
                maxlen = max(maxlen, len[g]);
            }
        }
        for (uint32_t q = 0; q < maxlen; ++q) {
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const int i = i0 + g;
                if (q < len[g]) {
                    const uint32_t kq = sm.keys[beg[g] + q];
                    if constexpr (PACKED) {
                        r[g] += kq < key[i] ? 1u : 0u;
                    } else {
                        r[g] += (kq < key[i] || (kq == key[i] && sm.seqs[beg[g] + q] < sqv[i])) ? 1u : 0u;
                    }
                }
            }
        }
#pragma unroll
        for (int g = 0; g < G; ++g) dst[i0 + g] = beg[g] + r[g];
    }
    row_sync<W>();
    // 7. products at their sorted positions
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const int p = (warp * ITEMS + i) * 32 + lane;
        if (p < P) {
            sm.keys[dst[i]] = key[i];
            if constexpr (!PACKED) sm.seqs[dst[i]] = static_cast<uint16_t>(sqv[i]);
        }
    }
    row_sync<W>();
    return true;
}


// The stable LSD radix sort of a row's products by column: 8-bit digits over
// the bits of max(col) - min(col), and with kNarrow a last pass of at most 4
// bits (four votes, 16 counters per warp) when no more remain.  Leaves keys
// (and seqs when !PACKED) in the layout finish_row reads.
template <int W, int ITEMS, bool SV, bool PACKED, bool kNarrow>
__device__ __forceinline__ void radix_sort_row(RowSmem<W, ITEMS, SV>& sm, int P, uint32_t cmin, int nbits, int lane,
                                               int warp, int tid) {
    constexpr int kSeqBits = RowSmem<W, ITEMS, SV>::kSeqBits;
    int hb = 0;  // counter set of this pass
    auto digits_from = [&](int shift) { return (kNarrow && nbits - shift <= 4) ? 16 : 256; };
    if constexpr (PACKED) {
        if (nbits == 0) {  // one column: already in sequence order; just pack
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const int pos = (warp * ITEMS + i) * 32 + lane;
                if (pos < P) sm.keys[pos] = ((sm.keys[pos] - cmin) << kSeqBits) | static_cast<uint32_t>(pos);
            }
        }
    } else {
        for (int i = tid; i < P; i += W * 32) sm.seqs[i] = static_cast<uint16_t>(i);
    }
    if (nbits > 0) clear_counters<W>(sm.hist[0], digits_from(0), tid);
    row_sync<W>();
    // One pass over the digit of NB bits at `shift` (NB = 8, or 4 for the last).
    auto pass = [&](auto nb, int shift) {
        constexpr int NB = decltype(nb)::value;
        constexpr uint32_t kMask = (1u << NB) - 1u;
        uint32_t* hist = sm.hist[hb];
        uint32_t k[ITEMS], rk[ITEMS];
        if constexpr (PACKED) {
            // Packed words (col - cmin) << kSeqBits | seq; the first pass packs.
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const int pos = (warp * ITEMS + i) * 32 + lane;
                uint32_t d = kMask;
                k[i] = 0xffffffffu;
                if (pos < P) {
                    const uint32_t raw = sm.keys[pos];
                    k[i] = shift == 0 ? ((raw - cmin) << kSeqBits) | static_cast<uint32_t>(pos) : raw;
                    d = (k[i] >> (kSeqBits + shift)) & kMask;
                }
                rk[i] = rank_item<NB>(d, &hist[hidx<W>(d, warp)], lane);
            }
            row_sync<W>();
            scan_counters<W, (1 << NB)>(hist, sm.warp_tmp);
            row_sync<W>();
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                // Padding items were ranked under the largest digit, after every
                // real item of that digit; they are not stored.
                const int pos = (warp * ITEMS + i) * 32 + lane;
                if (pos < P) {
                    const uint32_t d = (k[i] >> (kSeqBits + shift)) & kMask;
                    sm.keys[hist[hidx<W>(d, warp)] + rk[i]] = k[i];
                }
            }
        } else {
            uint16_t sq[ITEMS];
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const int pos = (warp * ITEMS + i) * 32 + lane;
                const bool valid = pos < P;
                k[i] = valid ? sm.keys[pos] : 0u;
                sq[i] = valid ? sm.seqs[pos] : uint16_t{0};
                const uint32_t d = valid ? (((k[i] - cmin) >> shift) & kMask) : kMask;
                rk[i] = rank_item<NB>(d, &hist[hidx<W>(d, warp)], lane);
            }
            row_sync<W>();
            scan_counters<W, (1 << NB)>(hist, sm.warp_tmp);
            row_sync<W>();
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const int pos = (warp * ITEMS + i) * 32 + lane;
                const uint32_t d = pos < P ? (((k[i] - cmin) >> shift) & kMask) : kMask;
                const uint32_t dst = hist[hidx<W>(d, warp)] + rk[i];
                if (dst < static_cast<uint32_t>(P)) {
                    sm.keys[dst] = k[i];
                    sm.seqs[dst] = sq[i];
                }
            }
        }
    };
    for (int shift = 0; shift < nbits;) {
        if (!kNarrow || nbits - shift > 4) {
            pass(std::integral_constant<int, 8>{}, shift);
            shift += 8;
        } else {
            if constexpr (kNarrow) pass(std::integral_constant<int, 4>{}, shift);
            shift += 4;
        }
        const bool more = shift < nbits;
        if constexpr (W == 1) {
            __syncwarp();
            if (more) clear_counters<W>(sm.hist[0], digits_from(shift), tid);
        } else if constexpr (kHistSets == 2) {
            if (more) clear_counters<W>(sm.hist[hb ^ 1], digits_from(shift), tid);
            hb ^= 1;
        } else {
            __syncthreads();  // the scatter above still reads the counters
            if (more) clear_counters<W>(sm.hist[0], digits_from(shift), tid);
        }
        row_sync<W>();
    }

}

// The radix sort of CTA rows that the bucket sort declined (a column repeated
// more than kMaxFine times): rare, so it keeps the code small rather than fast
// -- one key layout (columns and sequence numbers) and 8-bit digits only, then
// the packed words when the row's layout is packed.  Less code in the CTA
// kernels measured 0.25 ms faster on the power-law product than the full radix
// sort inline.
template <int W, int ITEMS, bool SV, bool PACKED>
__device__ __forceinline__ void radix_sort_fallback(RowSmem<W, ITEMS, SV>& sm, int P, uint32_t cmin, int nbits,
                                                    int lane, int warp, int tid) {
    constexpr int kSeqBits = RowSmem<W, ITEMS, SV>::kSeqBits;
    radix_sort_row<W, ITEMS, SV, false, false>(sm, P, cmin, nbits, lane, warp, tid);
    if constexpr (PACKED) {
        for (int i = tid; i < P; i += W * 32) sm.keys[i] = ((sm.keys[i] - cmin) << kSeqBits) | sm.seqs[i];
        row_sync<W>();  // a warp row's team is its warp: never a CTA barrier there
    }
}

// Steps 2-4 of a row for one key layout (PACKED: (col - cmin) << kSeqBits | seq
// words; otherwise columns and 16-bit sequence numbers).  Returns the stored
// entries this thread accounts for (its warp's on lane 0 in upper-bound mode,
// the row's on thread 0 in exact mode, else 0).  No barrier ends the row: the
// next row's enumeration passes a barrier before it writes what this phase
// reads (keys, values, sequence numbers, kept counts).
template <int W, int ITEMS, bool SV, bool PACKED>
__device__ uint32_t finish_row(const RowOut& out, RowSmem<W, ITEMS, SV>& sm, double* vals, int P, uint32_t cmin,
                           int nbits, int lane, int warp, int tid) {
    using Sm = RowSmem<W, ITEMS, SV>;
    constexpr int kSeqBits = Sm::kSeqBits;
    // 2. sort by column: the bucket sort for CTA rows, the radix sort for warp
    //    rows and where the bucket sort declines
    if constexpr (!kBucketRows<W, ITEMS>) {
        radix_sort_row<W, ITEMS, SV, PACKED, true>(sm, P, cmin, nbits, lane, warp, tid);
    } else {
        if (nbits == 0 || !bucket_sort<W, ITEMS, SV, PACKED>(sm, P, cmin, nbits, lane, warp, tid))
            radix_sort_fallback<W, ITEMS, SV, PACKED>(sm, P, cmin, nbits, lane, warp, tid);
    }

    // Column and sequence number of sorted position pos.
    auto col_at = [&](int pos) -> uint32_t {
        return PACKED ? (sm.keys[pos] >> kSeqBits) : sm.keys[pos] - cmin;
    };
    auto seq_at = [&](int pos) -> uint32_t {
        return PACKED ? (sm.keys[pos] & ((1u << kSeqBits) - 1u)) : sm.seqs[pos];
    };

    if (out.holes) {
        // 3+4 in one pass (upper-bound mode): sorted position pos owns slot
        // out0 + pos of the row's reserved range; the first position of every run
        // writes (column, sum) when the sum is != 0, every other slot column -1.
        const int64_t out0 = out.out0;
        uint32_t kept = 0;
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const int pos = (warp * ITEMS + i) * 32 + lane;
            if (pos < P) {
                const uint32_t c = col_at(pos);
                int32_t oc = -1;
                double acc = 0.0;
                if (pos == 0 || col_at(pos - 1) != c) {
                    acc = vals[seq_at(pos)];
                    for (int q = pos + 1; q < P && col_at(q) == c; ++q) acc = __dadd_rn(acc, vals[seq_at(q)]);
                    if (acc != 0.0) {
                        oc = static_cast<int32_t>(c + cmin);
                        ++kept;
                    }
                }
                out.c_col[out0 + pos] = oc;
                if (oc >= 0) out.c_val[out0 + pos] = acc;
            }
        }
        kept = __reduce_add_sync(0xffffffffu, kept);
        if (W == 1) {
            if (lane == 0) *out.nz = kept;
        } else if (lane == 0 && kept) {  // the row's count was zeroed before its enumeration
            atomicAdd(reinterpret_cast<unsigned long long*>(out.nz), static_cast<unsigned long long>(kept));
        }
        return lane == 0 ? kept : 0u;
    }

    // 3. runs of equal columns summed in product order; each run's sum is stored
    //    in place of its first product's value
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const int pos = (warp * ITEMS + i) * 32 + lane;
        bool keep = false;
        if (pos < P) {
            const uint32_t c = col_at(pos);
            if (pos == 0 || col_at(pos - 1) != c) {
                const uint32_t s0 = seq_at(pos);
                double acc = vals[s0];
                for (int q = pos + 1; q < P && col_at(q) == c; ++q) acc = __dadd_rn(acc, vals[seq_at(q)]);
                vals[s0] = acc;
                keep = acc != 0.0;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) sm.cnt[warp * ITEMS + i] = __popc(m);
    }
    row_sync<W>();
    scan_kept<W, ITEMS>(sm.cnt, sm.red, warp, lane);
    row_sync<W>();

    // 4. kept (column, sum) pairs in sorted order
    const int64_t out0 = out.out0;
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const int pos = (warp * ITEMS + i) * 32 + lane;
        bool keep = false;
        uint32_t c = 0;
        double v = 0.0;
        if (pos < P) {
            c = col_at(pos);
            if (pos == 0 || col_at(pos - 1) != c) {
                v = vals[seq_at(pos)];
                keep = v != 0.0;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const int64_t idx = out0 + sm.cnt[warp * ITEMS + i] + __popc(m & lanemask_lt());
            out.c_col[idx] = static_cast<int32_t>(c + cmin);
            out.c_val[idx] = v;
        }
    }
    if (tid == 0) *out.nz = sm.red[0];
    if constexpr (W == 1) __syncwarp();
    return tid == 0 ? static_cast<uint32_t>(sm.red[0]) : 0u;
}


// A column range of a split row: the products with columns in [lo, hi), which
// own slots [slot_off, slot_off + count) of the row's reserved range.  The
// row's products are staged in product order at scol / sval.
struct Piece {
    int64_t item;
    int32_t lo, hi;
    int64_t slot_off;
    int64_t count;
    const int32_t* scol;
    const double* sval;
};

// One row (PIECE = false) or one column range of a row (PIECE = true, CTA
// rows in upper-bound mode only).  Returns the stored entries this thread
// accounts for (finish_row).
template <int W, int ITEMS, bool SV, bool PIECE = false>
__device__ uint32_t numeric_row(const Job& J, int row, RowSmem<W, ITEMS, SV>& sm, double* vals, ErrWord* err,
                            const Piece* pc = nullptr) {
    using Sm = RowSmem<W, ITEMS, SV>;
    constexpr int kSeqBits = Sm::kSeqBits;
    const int lane = threadIdx.x & 31;
    const int warp = W == 1 ? 0 : (threadIdx.x >> 5);
    const int tid = W == 1 ? lane : threadIdx.x;
    const int P = static_cast<int>(PIECE ? pc->count : J.ub[row]);
    if constexpr (W > 1) {
        // an upper-bound row's warps add their kept counts to its count after the
        // barriers below (a piece's row count was zeroed by the planner)
        if (!PIECE && J.holes && tid == 0) J.nz[row] = 0;
    }
    if constexpr (kBucketRows<W, ITEMS>) clear_buckets(sm, P, tid);

    // 1. products into shared memory
    int32_t lo = INT32_MAX, hi = INT32_MIN;
    const int32_t ncols = J.B.cols;
    auto put = [&](int32_t seq, int32_t c, double prod) {
        if (PIECE && seq >= P) {  // the planner counted fewer products in this range: never writes past P
            raise_error(err, kErrInvalid, 8, seq);
            return;
        }
        if (c < 0 || c >= ncols) {
            raise_error(err, kErrInvalid, 4, c);
            c = 0;
        }
        sm.keys[seq] = static_cast<uint32_t>(c);
        vals[seq] = prod;
        lo = min(lo, c);
        hi = max(hi, c);
    };
    if constexpr (PIECE)
        staged_products_in<W * 32>(pc->scol, pc->sval, static_cast<int32_t>(J.ub[row]), sm.step_cnt, tid, pc->lo,
                                   pc->hi, put);
    else
        team_row_products<W * 32, Sm::kCap>(J, row, sm.seg, sm.warp_tmp, tid,
                                            [&](int32_t seq, int32_t c, double b, double a) {
                                                put(seq, c, __dmul_rn(a, b));
                                            });
    lo = __reduce_min_sync(0xffffffffu, lo);  // one warp-wide reduction instruction each
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (W > 1) {
        if (lane == 0) {
            sm.red[warp] = lo;
            sm.red[W + warp] = hi;
        }
        __syncthreads();
        lo = sm.red[0];
        hi = sm.red[W];
#pragma unroll
        for (int w = 1; w < W; ++w) {
            lo = min(lo, sm.red[w]);
            hi = max(hi, sm.red[W + w]);
        }
    } else {
        __syncwarp();  // the enumeration's last batch ends without one
    }
    const uint32_t cmin = static_cast<uint32_t>(lo);
    const uint32_t range = P ? static_cast<uint32_t>(hi - lo) : 0u;
    const int nbits = range ? 32 - __clz(range) : 0;
    const RowOut out{J.c_col, J.c_val, J.cnt[row] + (PIECE ? pc->slot_off : 0), J.nz + row, J.holes, PIECE ? 1 : 0};
    if (nbits + kSeqBits <= 32) return finish_row<W, ITEMS, SV, true>(out, sm, vals, P, cmin, nbits, lane, warp, tid);
    return finish_row<W, ITEMS, SV, false>(out, sm, vals, P, cmin, nbits, lane, warp, tid);
}

constexpr int kWarpKernelThreads = 256;

// Resident CTAs per SM the warp-row kernels are compiled for (caps registers
// at 80 and 64 per thread).  Measured on power-law rows, one bin at a time:
// the 12- and 16-item kernels 0.92 / 0.85 -> 0.79 / 0.80 ms against 2 CTAs
// (128 registers), the 6- and 8-item ones 0.39 -> 0.35 ms against 3.
constexpr int warp_kernel_min_blocks(int items) { return items >= 12 ? 3 : 4; }

// The row kernels are persistent: a launch has at most a few waves of CTAs
// that loop over the bin's rows.  A warp-row kernel takes its rows by a fixed
// stride: its rows are many and light, and a ticket per row measured 4% slower
// on the uniform product (one counter for hundreds of thousands of rows).
template <int ITEMS>
__global__ void __launch_bounds__(kWarpKernelThreads, warp_kernel_min_blocks(ITEMS))
num_warp_kernel(const Job* __restrict__ jobs, const int64_t* __restrict__ items, int64_t count,
                Stats* __restrict__ stats, ErrWord* __restrict__ err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Sm = RowSmem<1, ITEMS>;
    Sm& sm = reinterpret_cast<Sm*>(smem_raw)[threadIdx.x >> 5];
    __shared__ unsigned long long s_nz;
    if (threadIdx.x == 0) s_nz = 0;
    __syncthreads();
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (kWarpKernelThreads / 32);
    unsigned long long mine = 0;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * (kWarpKernelThreads / 32) + (threadIdx.x >> 5); i < count;
         i += warps) {
        const int64_t it = items[i];
        const Job& J = jobs[item_job(it)];
        const int row = item_row(it);
        mine += numeric_row<1, ITEMS, true>(J, row, sm, sm.vals, err);
    }
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&s_nz, mine);
    __syncthreads();
    if (threadIdx.x == 0 && s_nz) atomicAdd(&stats->nz_total, s_nz);
}

// A CTA-row kernel (and the split rows' pieces) pulls its rows from the
// launch's row queue: the CTA's first row is its index, each later one
// gridDim.x plus the next ticket of the bin's counter, so that rows of very
// different cost spread over the CTAs as they free up.  Thread 0 fetches the
// ticket at the start of the current row (the other warps start on the row
// meanwhile; fetching it a row ahead instead, in a register, measured slower)
// into one of two shared words (alternating rows); every thread reads it after
// the row, whose barriers order the store before the reads, and every read
// before the store two rows later.
struct RowQueue {
    int64_t next[2];
};

template <int W, int ITEMS, int MINB, bool SV>
__global__ void __launch_bounds__(W * 32, MINB)
num_block_kernel(const Job* __restrict__ jobs, const int64_t* __restrict__ items, int64_t count,
                 Stats* __restrict__ stats, ErrWord* __restrict__ err, double* __restrict__ gvals,
                 unsigned long long* __restrict__ ticket) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ RowQueue q;
    using Sm = RowSmem<W, ITEMS, SV>;
    Sm& sm = *reinterpret_cast<Sm*>(smem_raw);
    double* vals = SV ? sm.vals : gvals + static_cast<size_t>(blockIdx.x) * Sm::kCap;
    unsigned long long mine = 0;
    int par = 0;
    for (int64_t i = blockIdx.x; i < count; par ^= 1) {
        if (threadIdx.x == 0)
            q.next[par] = static_cast<int64_t>(gridDim.x) + static_cast<int64_t>(atomicAdd(ticket, 1ull));
        const int64_t it = items[i];
        const Job& J = jobs[item_job(it)];
        const int row = item_row(it);
        mine += numeric_row<W, ITEMS, SV>(J, row, sm, vals, err);
        i = q.next[par];
    }
    if (mine) atomicAdd(&stats->nz_total, mine);
}

inline int capped(int64_t work, int per_block, int cap) {
    const int64_t g = (work + per_block - 1) / per_block;
    return static_cast<int>(g < 1 ? 1 : (g > cap ? cap : g));
}

// CTAs of a launch whose CTAs each own a global slab: minb per SM at most.
inline int slab_grid(int64_t count, int num_sms, int minb = 1) {
    const int64_t cap = static_cast<int64_t>(num_sms) * minb;
    return static_cast<int>(count < cap ? count : cap);
}

template <int ITEMS>
void run_warp(const Job* jobs, const int64_t* items, int64_t count, Stats* stats, ErrWord* err, cudaStream_t st,
              int num_sms) {
    const int smem = 8 * static_cast<int>(sizeof(RowSmem<1, ITEMS>));
    cudaFuncSetAttribute(num_warp_kernel<ITEMS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    num_warp_kernel<ITEMS><<<capped(count, 8, num_sms * 16), kWarpKernelThreads, smem, st>>>(jobs, items, count, stats,
                                                                                           err);
}

template <int W, int ITEMS, int MINB, bool SV = true>
void run_block(const Job* jobs, const int64_t* items, int64_t count, Stats* stats, ErrWord* err, cudaStream_t st,
               int num_sms, unsigned long long* ticket, double* gvals = nullptr) {
    const int smem = static_cast<int>(sizeof(RowSmem<W, ITEMS, SV>));
    cudaFuncSetAttribute(num_block_kernel<W, ITEMS, MINB, SV>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    // One wave of resident CTAs: with the row queue, CTAs beyond it would start
    // only once the queue has run dry (slab bins: one slab per resident CTA).
    static std::atomic<int> resident{0};  // per instantiation (every device of this build is an sm_103a)
    int nb = resident.load(std::memory_order_relaxed);
    if (nb == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, num_block_kernel<W, ITEMS, MINB, SV>, W * 32, smem) !=
                cudaSuccess || nb < 1) {
            cudaGetLastError();
            nb = MINB;
        }
        resident.store(nb, std::memory_order_relaxed);
    }
    const int grid = SV ? capped(count, 1, num_sms * nb) : slab_grid(count, num_sms, MINB);
    num_block_kernel<W, ITEMS, MINB, SV><<<grid, W * 32, smem, st>>>(jobs, items, count, stats, err, gvals, ticket);
}

}  // namespace
}  // namespace spg
