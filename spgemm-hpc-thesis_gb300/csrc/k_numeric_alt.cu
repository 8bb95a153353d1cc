// K4 numeric phase: the alternative team shape of each bin that has one, for
// the autotuner (spg_tune).  Every shape runs the same per-row pipeline
// (k_numeric_row.cuh), so results are identical; only the time differs.
//   bins 7-8   (<= 384, <= 512 products): a 2-warp CTA per row instead of one warp
//   bins 9-15  (<= 768 ... <= 6144):      the shapes before the last measurement-driven tuning
//   bins 17-18 (<= 12288, <= 16384):      whole rows, one 16-warp CTA each, instead of
//                                         column-range pieces (upper-bound layout; k_numeric.cu)
#include "k_numeric_row.cuh"

namespace spg {

bool launch_numeric_alt(int bin, const Job* d_jobs, const int64_t* d_items, int64_t count, Stats* d_stats,
                        ErrWord* d_err, cudaStream_t st, int num_sms) {
    unsigned long long* const tk = &d_stats->ticket[bin];  // the bin's row queue
    switch (bin) {
        case 7: run_block<2, 6, 8>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); return true;    // 384
        case 8: run_block<2, 8, 8>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); return true;    // 512
        case 9: run_block<3, 8, 8>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); return true;    // 768
        case 10: run_block<4, 8, 6>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); return true;   // 1024
        case 11: run_block<8, 6, 4>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); return true;   // 1536
        case 12: run_block<4, 16, 4>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); return true;  // 2048
        case 13: run_block<8, 12, 2>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); return true;  // 3072
        case 14: run_block<16, 8, 1>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); return true;  // 4096
        case 15: run_block<12, 16, 1>(d_jobs, d_items, count, d_stats, d_err, st, num_sms, tk); return true; // 6144
        default: return false;
    }
}

}  // namespace spg
