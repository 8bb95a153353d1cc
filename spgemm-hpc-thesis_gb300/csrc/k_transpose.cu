// CSR transpose on the GPU: A^T keeps, in every row, the entries of A's
// column in A's row-major order (a stable counting sort by column), which is
// what a transposition by stable sort of the entries produces on the host.
//
// A device-wide stable LSD radix sort of the entry indices by column, 8-bit
// digits over the bits of (cols - 1).  Each pass: per-tile digit histograms
// (tile = 8192 entries), one scan of the digit-major (digit, tile) table, and
// a scatter in which every tile ranks its entries stably with the warp ballot
// groups and per-warp digit counters of the numeric kernels.
#include "k_numeric_row.cuh"

namespace spg {
namespace {

constexpr int kTW = 16;
constexpr int kTItems = 16;
constexpr int kTThreads = kTW * 32;
constexpr int kTTile = kTThreads * kTItems;

// row index of every entry (warp per row)
__global__ void expand_rows_kernel(const int64_t* __restrict__ rp, int32_t rows, int32_t* __restrict__ row_of) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x / 32);
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5); r < rows; r += warps)
        for (int64_t p = rp[r] + lane; p < rp[r + 1]; p += 32) row_of[p] = static_cast<int32_t>(r);
}

__global__ void iota_kernel(int64_t* __restrict__ idx, int64_t n) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        idx[i] = i;
}

// counts[d * tiles + tile] of digit d in each tile
__global__ void __launch_bounds__(kTThreads)
tile_hist_kernel(const int32_t* __restrict__ col, const int64_t* __restrict__ idx, int64_t n, int shift,
                 int64_t tiles, int64_t* __restrict__ counts) {
    __shared__ uint32_t h[256];
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        if (threadIdx.x < 256) h[threadIdx.x] = 0;
        __syncthreads();
        const int64_t t0 = tile * kTTile;
        for (int i = threadIdx.x; i < kTTile; i += kTThreads) {
            const int64_t p = t0 + i;
            if (p < n) atomicAdd(&h[(static_cast<uint32_t>(col[idx[p]]) >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x < 256) counts[static_cast<int64_t>(threadIdx.x) * tiles + tile] = h[threadIdx.x];
        __syncthreads();
    }
}

struct TileSmem {
    uint32_t hist[kHistWords<kTW>];
    int64_t warp_tmp[kTW + 1];
};

// Stable scatter of one pass: entry i of the tile (striped order = input
// order) goes to offs[d * tiles + tile] + (its rank among the tile's entries of
// digit d).
__global__ void __launch_bounds__(kTThreads)
tile_scatter_kernel(const int32_t* __restrict__ col, const int64_t* __restrict__ idx_in, int64_t* __restrict__ idx_out,
                    int64_t n, int shift, int64_t tiles, const int64_t* __restrict__ offs) {
    __shared__ TileSmem sm;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        for (int d = threadIdx.x; d < kHistWords<kTW>; d += kTThreads) sm.hist[d] = 0;
        __syncthreads();
        const int64_t t0 = tile * kTTile;
        int64_t v[kTItems];
        uint32_t rk[kTItems];
#pragma unroll
        for (int i = 0; i < kTItems; ++i) {
            const int64_t p = t0 + (warp * kTItems + i) * 32 + lane;
            uint32_t d = 255u;
            v[i] = -1;
            if (p < n) {
                v[i] = idx_in[p];
                d = (static_cast<uint32_t>(col[v[i]]) >> shift) & 255u;
            }
            rk[i] = rank_item(d, &sm.hist[hidx<kTW>(d, warp)], lane);
        }
        __syncthreads();
        scan_counters<kTW>(sm.hist, sm.warp_tmp);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < kTItems; ++i) {
            if (v[i] < 0) continue;  // padding past the end (ranked last under digit 255)
            const uint32_t d = (static_cast<uint32_t>(col[v[i]]) >> shift) & 255u;
            const uint32_t within = sm.hist[hidx<kTW>(d, warp)] + rk[i] - sm.hist[hidx<kTW>(d, 0)];
            idx_out[offs[static_cast<int64_t>(d) * tiles + tile] + within] = v[i];
        }
        __syncthreads();
    }
}

__global__ void col_count_kernel(const int32_t* __restrict__ col, int64_t n, int64_t* __restrict__ cnt) {
    for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x)
        atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[col[p]]), 1ull);
}

__global__ void gather_t_kernel(const int64_t* __restrict__ perm, const int32_t* __restrict__ row_of,
                                const double* __restrict__ val, int64_t n, int32_t* __restrict__ out_col,
                                double* __restrict__ out_val) {
    for (int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
         q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t p = perm[q];
        out_col[q] = row_of[p];
        out_val[q] = val[p];
    }
}

int grid_of(int64_t work, int per_block, int cap) {
    const int64_t g = (work + per_block - 1) / per_block;
    return static_cast<int>(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

size_t transpose_scratch_bytes(int64_t nnz, int32_t cols) {
    const int64_t tiles = (nnz + kTTile - 1) / kTTile;
    return static_cast<size_t>(nnz) * (4 + 8 + 8) + static_cast<size_t>(256 * tiles + 1) * 8 +
           scan_partials_count(256 * tiles + 1) * 8 + static_cast<size_t>(cols + 1) * 8 + 4096;
}

// scratch: row_of (4 nnz) | idx A (8 nnz) | idx B (8 nnz) | counts (8 (256 tiles + 1)) | partials
void launch_transpose(const int64_t* rp, const int32_t* col, const double* val, int32_t rows, int32_t cols, int64_t nnz,
                      int64_t* out_rp, int32_t* out_col, double* out_val, void* scratch, cudaStream_t st) {
    const int64_t tiles = (nnz + kTTile - 1) / kTTile;
    auto up = [](size_t x) { return (x + 255) & ~size_t{255}; };
    unsigned char* s = static_cast<unsigned char*>(scratch);
    int32_t* row_of = reinterpret_cast<int32_t*>(s);
    size_t o = up(static_cast<size_t>(nnz) * 4);
    int64_t* ia = reinterpret_cast<int64_t*>(s + o);
    o = up(o + static_cast<size_t>(nnz) * 8);
    int64_t* ib = reinterpret_cast<int64_t*>(s + o);
    o = up(o + static_cast<size_t>(nnz) * 8);
    int64_t* counts = reinterpret_cast<int64_t*>(s + o);
    o = up(o + static_cast<size_t>(256 * tiles + 1) * 8);
    int64_t* partials = reinterpret_cast<int64_t*>(s + o);

    // row pointer of A^T: column counts, scanned
    cudaMemsetAsync(out_rp, 0, sizeof(int64_t) * (static_cast<size_t>(cols) + 1), st);
    if (nnz > 0) col_count_kernel<<<grid_of(nnz, 256, 152 * 16), 256, 0, st>>>(col, nnz, out_rp);
    launch_scan(out_rp, cols, partials, st);
    if (nnz == 0) return;
    expand_rows_kernel<<<grid_of(rows, 8, 152 * 16), 256, 0, st>>>(rp, rows, row_of);
    iota_kernel<<<grid_of(nnz, 256, 152 * 16), 256, 0, st>>>(ia, nnz);
    int bits = 0;
    while (bits < 31 && (int64_t{1} << bits) < cols) ++bits;
    const int grid = grid_of(tiles, 1, 152 * 4);
    for (int shift = 0; shift < bits; shift += 8) {
        tile_hist_kernel<<<grid, kTThreads, 0, st>>>(col, ia, nnz, shift, tiles, counts);
        cudaMemsetAsync(counts + 256 * tiles, 0, sizeof(int64_t), st);
        launch_scan(counts, 256 * tiles, partials, st);
        tile_scatter_kernel<<<grid, kTThreads, 0, st>>>(col, ia, ib, nnz, shift, tiles, counts);
        std::swap(ia, ib);
    }
    gather_t_kernel<<<grid_of(nnz, 256, 152 * 16), 256, 0, st>>>(ia, row_of, val, nnz, out_col, out_val);
}

}  // namespace spg
