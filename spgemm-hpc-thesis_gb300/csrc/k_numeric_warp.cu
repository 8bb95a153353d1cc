// K4 numeric phase: the row bins that run one row per warp (<= 512 products;
// 1, 2, 3, 4, 6, 8, 12 or 16 products per lane).  The per-row pipeline is in
// k_numeric_row.cuh; this translation unit only instantiates it, so that it
// compiles in parallel with the CTA-per-row bins.
#include "k_numeric_row.cuh"

namespace spg {

void launch_numeric_warp(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, Stats* d_stats,
                         ErrWord* d_err, cudaStream_t st, int num_sms) {
    switch (bin) {
        case 1: run_warp<1>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;
        case 2: run_warp<2>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;
        case 3: run_warp<3>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;
        case 4: run_warp<4>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;
        case 5: run_warp<6>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;
        case 6: run_warp<8>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;
        case 7: run_warp<12>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;
        case 8: run_warp<16>(d_jobs, d_items, count, d_stats, d_err, st, num_sms); break;
        default: break;
    }
}

}  // namespace spg
