// Enumeration of the scalar products of one output row in the reference order.
//
// A row's products are the concatenation of "segments": the addend row S_i
// (scale 1.0) when present, then, for every A entry (k, a) in stored order, the
// B row k scaled by a.  Product number t of the row (its sequence number) is
// the t-th element of that concatenation, which is the order in which
// serialSpgemm (spgemm_common.cpp:139-152) and spgemm() (spgemm_exchange.cpp:
// 279-294) visit them.
//
// Segments are processed in batches of one per thread: the batch's segment
// lengths are scanned and its descriptors staged in shared memory.  The team's
// threads then stride over the batch's products (neighbouring threads read
// neighbouring B entries, coalesced), U products per thread at a time (four by
// default): each finds its segment by binary search, then their column and
// value loads are issued together, so a thread keeps 2U independent global
// loads in flight instead of one.
#pragma once

#include "spg_common.cuh"

namespace spg {

// Idx is int32_t for rows of at most 2^31 - 1 products (every shared-memory
// path), int64_t otherwise.
__host__ __device__ constexpr int pow2_ceil_c(int x) { return x <= 1 ? 1 : 2 * pow2_ceil_c((x + 1) / 2); }

template <int N, typename Idx = int64_t>
struct SegTab {
    static constexpr int kPad = pow2_ceil_c(N) - N;  // entries past N, above every sequence number
    const int32_t* colp[N];
    const double* valp[N];
    double scale[N];
    Idx incl[N + kPad];  // inclusive prefix of segment lengths within the batch
};

// Writes the padding entries of a team's segment table (once per enumeration).
template <int N, typename Idx>
__device__ inline void pad_segtab(SegTab<N, Idx>& tab, int tid) {
    if (SegTab<N, Idx>::kPad && tid < SegTab<N, Idx>::kPad) tab.incl[N + tid] = static_cast<Idx>(INT64_MAX >> (64 - 8 * sizeof(Idx)));
}

// Segment e of a row (e counts the addend first when present).
template <typename Idx>
__device__ inline void row_segment(const Job& J, int row, int64_t a0, bool has_s, int64_t e,
                                   const int32_t*& cp, const double*& vp, double& sc, Idx& len) {
    if (has_s && e == 0) {
        const int64_t s0 = J.S.rp[row];
        cp = J.S.ci + s0;
        vp = J.S.v + s0;
        sc = 1.0;
        len = static_cast<Idx>(J.S.rp[row + 1] - s0);
    } else {
        const int64_t p = a0 + e - (has_s ? 1 : 0);
        const int32_t k = J.A.ci[p];
        const int64_t b0 = J.B.rp[k];
        cp = J.B.ci + b0;
        vp = J.B.v + b0;
        sc = J.A.v[p];
        len = static_cast<Idx>(J.B.rp[k + 1] - b0);
    }
}

// Smallest j in [0, N) with incl[j] > t (the batch total exceeds t): the
// number of entries <= t, by binary lifting over the next power of two.  The
// table's padding entries (pad_segtab) exceed every t, so no step needs a
// bound test.
template <int N, typename Idx>
__device__ inline int seg_search(const Idx* incl, Idx t) {
    int j = 0;
#pragma unroll
    for (int step = pow2_ceil_c(N) / 2; step >= 1; step >>= 1)
        if (incl[j + step - 1] <= t) j += step;
    return j;
}

// Inclusive block scan (NT threads, NT/32 <= 32 warps).
template <int NT, typename Idx>
__device__ inline Idx block_incl_scan(Idx v, int64_t* s_warp /* NT/32 + 1 */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int NW = NT / 32;
    const Idx incl = warp_incl_scan(v, lane);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const Idx w = lane < NW ? static_cast<Idx>(s_warp[lane]) : Idx{0};
        const Idx wi = warp_incl_scan(w, lane);
        if (lane < NW) s_warp[lane] = wi - w;
    }
    __syncthreads();
    const Idx out = incl + static_cast<Idx>(s_warp[warp]);
    __syncthreads();
    return out;
}

template <int NT>
__device__ inline void team_sync() {
    if (NT == 32) __syncwarp();
    else __syncthreads();
}

// Team-cooperative enumeration: a warp (NT == 32, tid = lane) or a whole CTA
// (NT == blockDim.x, tid = threadIdx.x); every thread of the team must call it.
// f(seq, col, b, a) is called once per product by the thread that owns it, with
// the B entry's column `col`, its value `b` and the scale `a` (the product is
// a*b).  kLoadVal = false skips the value loads (b is then 0).  Idx is the
// index type of sequence numbers within the row (int32_t when the row has fewer
// than 2^31 products, which keeps the per-product search in 32-bit integers).
// U products per thread are resolved and loaded together.
template <int NT, bool kLoadVal, typename Idx = int64_t, int U = 4, typename F>
__device__ inline void team_products(const Job& J, int row, SegTab<NT, Idx>& tab, int64_t* s_warp, int tid,
                                     F&& f) {
    const bool has_s = J.S.rp != nullptr;
    const int64_t a0 = J.A.rp[row];
    const int64_t nseg = (J.A.rp[row + 1] - a0) + (has_s ? 1 : 0);
    pad_segtab(tab, tid);
    Idx seq_base = 0;
    for (int64_t e0 = 0; e0 < nseg; e0 += NT) {
        const int64_t e = e0 + tid;
        const int32_t* cp = nullptr;
        const double* vp = nullptr;
        double sc = 1.0;
        Idx len = 0;
        if (e < nseg) row_segment(J, row, a0, has_s, e, cp, vp, sc, len);
        Idx incl;
        if constexpr (NT == 32) incl = warp_incl_scan(len, tid);
        else incl = block_incl_scan<NT>(len, s_warp);
        tab.colp[tid] = cp;
        tab.valp[tid] = vp;
        tab.scale[tid] = sc;
        tab.incl[tid] = incl;
        team_sync<NT>();
        const Idx total = tab.incl[NT - 1];
        for (Idx t0 = tid; t0 < total; t0 += U * NT) {
            int j[U];
            Idx q[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const Idx t = t0 + u * NT;
                j[u] = t < total ? seg_search<NT>(tab.incl, t) : 0;
                q[u] = t < total ? t - (j[u] ? tab.incl[j[u] - 1] : Idx{0}) : Idx{0};
            }
            int32_t c[U];
            double b[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool ok = t0 + u * NT < total;
                c[u] = ok ? __ldg(tab.colp[j[u]] + q[u]) : 0;
                b[u] = (kLoadVal && ok) ? __ldg(tab.valp[j[u]] + q[u]) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (t0 + u * NT < total) f(seq_base + t0 + u * NT, c[u], b[u], tab.scale[j[u]]);
        }
        seq_base += total;
        team_sync<NT>();
    }
}

// Segment table of team_row_products: rows of at most CAP products, NT
// segments per batch.  Entry r describes the r-th non-empty segment of the
// batch: the byte addresses of its B columns and values less 4 and 8 bytes
// times its first position in the batch (so product t of the batch lies at
// colb[r] + 4t, valb[r] + 8t), and its scale.  word[w] covers batch positions
// [32w, 32w + 32): x has bit b set where a non-empty segment starts at 32w + b,
// y is the rank r of the segment holding position 32w.
template <int NT, int CAP>
struct RowSegs {
    static_assert(CAP % 32 == 0 && CAP < 65536, "positions and non-empty counts share one 32-bit scan");
    uint64_t colb[NT];
    uint64_t valb[NT];
    double scale[NT];
    uint2 word[CAP / 32];
};

// team_products for rows of at most CAP products (every row the shared-memory
// row kernels take): the same products, sequence numbers and calls of f, but a
// product finds its segment from the batch's start mask (one broadcast load and
// a population count: the rank of the segment holding the word's first
// position plus the starts between that position and the product's) instead of
// a binary search over the batch's prefix sums.  t & 31 is the lane for every
// product a thread takes (the team strides by multiples of 32), so the mask bits
// at or below the product's position are lanemask_le.  The last batch ends
// without a barrier: the caller's next barrier (or, for a warp, __syncwarp)
// orders the products' shared-memory stores before their readers.
template <int NT, int CAP, int U = 4, typename F>
__device__ inline void team_row_products(const Job& J, int row, RowSegs<NT, CAP>& tab, int64_t* s_warp, int tid,
                                         F&& f) {
    const bool has_s = J.S.rp != nullptr;
    const int64_t a0 = J.A.rp[row];
    const int64_t nseg = (J.A.rp[row + 1] - a0) + (has_s ? 1 : 0);
    const int lane = tid & 31;
    const unsigned le_above0 = (lanemask_lt() | (1u << lane)) & ~1u;  // bits (0, lane]
    int32_t seq_base = 0;
    for (int64_t e0 = 0; e0 < nseg; e0 += NT) {
        const int64_t e = e0 + tid;
        const int32_t* cp = nullptr;
        const double* vp = nullptr;
        double sc = 1.0;
        int32_t len = 0;
        if (e < nseg) row_segment(J, row, a0, has_s, e, cp, vp, sc, len);
        // the start mask is cleared before the scan's barrier and set after it
        for (int w = tid; w < CAP / 32; w += NT) tab.word[w].x = 0u;
        if constexpr (NT == 32) __syncwarp();
        // low 16 bits: products; high 16 bits: non-empty segments.  One barrier:
        // every warp scans the warp totals itself (s_warp is rewritten only
        // after the batch's later barriers).
        const uint32_t packed = static_cast<uint32_t>(len) | (len > 0 ? 0x10000u : 0u);
        uint32_t incl = warp_incl_scan(packed, lane);
        uint32_t total_packed;
        if constexpr (NT == 32) {
            total_packed = __shfl_sync(0xffffffffu, incl, 31);
        } else {
            constexpr int NW = NT / 32;
            const int warp = tid >> 5;
            if (lane == 31) s_warp[warp] = incl;
            __syncthreads();
            const uint32_t wt = lane < NW ? static_cast<uint32_t>(s_warp[lane]) : 0u;
            const uint32_t wincl = warp_incl_scan(wt, lane);
            incl += __shfl_sync(0xffffffffu, wincl - wt, warp);
            total_packed = __shfl_sync(0xffffffffu, wincl, NW - 1);
        }
        if (len > 0) {
            const uint32_t s = (incl & 0xffffu) - static_cast<uint32_t>(len);
            const uint32_t r = (incl >> 16) - 1u;
            tab.colb[r] = reinterpret_cast<uint64_t>(cp) - 4u * static_cast<uint64_t>(s);
            tab.valb[r] = reinterpret_cast<uint64_t>(vp) - 8u * static_cast<uint64_t>(s);
            tab.scale[r] = sc;
            atomicOr(&tab.word[s >> 5].x, 1u << (s & 31u));
            for (uint32_t w = (s + 31u) >> 5; (w << 5) < s + static_cast<uint32_t>(len); ++w) tab.word[w].y = r;
        }
        team_sync<NT>();
        const int32_t total = static_cast<int32_t>(total_packed & 0xffffu);
        for (int32_t t0 = tid; t0 < total; t0 += U * NT) {
            int r[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int32_t t = t0 + u * NT;
                r[u] = 0;
                if (t < total) {
                    const uint2 wd = tab.word[t >> 5];
                    r[u] = static_cast<int>(wd.y) + __popc(wd.x & le_above0);
                }
            }
            int32_t c[U];
            double b[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int32_t t = t0 + u * NT;
                const bool ok = t < total;
                c[u] = ok ? __ldg(reinterpret_cast<const int32_t*>(tab.colb[r[u]] + 4u * static_cast<uint64_t>(t))) : 0;
                b[u] = ok ? __ldg(reinterpret_cast<const double*>(tab.valb[r[u]] + 8u * static_cast<uint64_t>(t))) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (t0 + u * NT < total) f(seq_base + t0 + u * NT, c[u], b[u], tab.scale[r[u]]);
        }
        seq_base += total;
        if (e0 + NT < nseg) team_sync<NT>();  // the next batch rewrites the table
    }
}

// The products of a staged row (columns scol[0..n), values sval[0..n), in the
// row's product order) whose column lies in [lo, hi), for a whole CTA (NT
// threads, 8 * NT/32 <= 64).  Kept products are numbered 0, 1, ... in row
// order, so a stable sort of the kept ones by column keeps the reference order
// of every column.  Each step of 8*NT products (coalesced loads, eight columns
// per thread in flight: the staging is mostly read from DRAM) compacts its
// kept flags with one ballot per product slot and a scan of the 8*(NT/32)
// warp counts (s_cnt, 64 words).  f(local_seq, col, product) is called once
// per kept product.
template <int NT, typename F>
__device__ inline void staged_products_in(const int32_t* __restrict__ scol, const double* __restrict__ sval,
                                          int32_t n, uint32_t* s_cnt, int tid, int32_t lo, int32_t hi, F&& f) {
    constexpr int NW = NT / 32;
    constexpr int U = 8;
    static_assert(U * NW <= 64, "at most 8 warps");
    const int lane = tid & 31, warp = tid >> 5;
    int32_t kept_base = 0;
    for (int32_t t0 = 0; t0 < n; t0 += U * NT) {  // uniform trip count: every thread reaches the barriers
        int32_t c[U];
        bool keep[U];
        unsigned m[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int32_t t = t0 + u * NT + tid;
            c[u] = t < n ? __ldg(scol + t) : 0;
        }
        double v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int32_t t = t0 + u * NT + tid;
            keep[u] = t < n && c[u] >= lo && c[u] < hi;
            v[u] = keep[u] ? __ldg(sval + t) : 0.0;
            m[u] = __ballot_sync(0xffffffffu, keep[u]);
            if (lane == 0) s_cnt[u * NW + warp] = static_cast<uint32_t>(__popc(m[u]));
        }
        __syncthreads();
        // exclusive scan of the U*NW counts in (u, warp) order, two per lane
        const uint32_t x0 = 2 * lane < U * NW ? s_cnt[2 * lane] : 0u;
        const uint32_t x1 = 2 * lane + 1 < U * NW ? s_cnt[2 * lane + 1] : 0u;
        const uint32_t pair_incl = warp_incl_scan(x0 + x1, lane);
        const uint32_t step_total = __shfl_sync(0xffffffffu, pair_incl, 31);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int idx = u * NW + warp;
            const uint32_t pi = __shfl_sync(0xffffffffu, pair_incl, idx >> 1);
            const uint32_t p0 = __shfl_sync(0xffffffffu, x0, idx >> 1);
            const uint32_t p1 = __shfl_sync(0xffffffffu, x1, idx >> 1);
            const uint32_t excl = (pi - p0 - p1) + ((idx & 1) ? p0 : 0u);
            if (keep[u]) f(kept_base + static_cast<int32_t>(excl + __popc(m[u] & lanemask_lt())), c[u], v[u]);
        }
        kept_base += static_cast<int32_t>(step_total);
        __syncthreads();  // s_cnt is rewritten by the next step
    }
}

__device__ inline uint32_t hash_slot(int32_t col, int log2t) {
    return (static_cast<uint32_t>(col) * 0x9E3779B1u) >> (32 - log2t);
}

__host__ __device__ inline int ceil_log2(int64_t x) {
    int l = 0;
    while ((int64_t{1} << l) < x) ++l;
    return l;
}

}  // namespace spg
