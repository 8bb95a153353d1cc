// Host side of the GB300 SpGEMM engine and its C ABI (include/spgemm_gb300.h).
//
// One call runs the phases on the handle's stream:
//   stage operands -> K1 row work + bins -> [sync: bin sizes, errors]
//   -> K2 symbolic per bin -> K3 scan -> [sync: C size] -> allocate C
//   -> K4 numeric per bin -> [sync: stored count, errors]
//   -> (K5 compaction only if some sum was an exact zero) -> result.
// All rows of all products of a call are flattened into one set of bin lists,
// so a batch of products costs the same number of launches as one product.
// Device memory comes from the device's stream-ordered pool (cudaMallocAsync),
// whose release threshold is raised so that repeated calls reuse memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <limits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/spgemm_gb300.h"
#include "spg_common.cuh"


using namespace spg;

struct spg_handle {
    int device = 0;
    int num_sms = 152;
    cudaStream_t stream = nullptr;
    spg_config cfg{};
    std::string err;
    cudaEvent_t ev[6] = {};
    cudaEvent_t bin_ev[kNumBins] = {};  // end of each bin's numeric launch
    // numeric bins run on three streams (warp bins on `stream`; shared-memory
    // CTA bins; slab and heavy bins, which share the scratch), so that one
    // launch's tail overlaps the others; fork/join events
    cudaStream_t aux[2] = {};
    cudaEvent_t fork = nullptr, join[2] = {};
    bool serial_bins = false;  // spg_tune times bins one after the other
    bool one_bin_stream = false;  // spg_config.bin_streams == 1
    spg_timings last{};
    // accumulate mode: the running sum S (device result) and its shape
    bool acc_active = false;
    int32_t acc_rows = 0, acc_cols = 0;
    spg_csr_result acc{};
    bool acc_has = false;
    // pinned control block for small device->host reads
    void* ctrl = nullptr;
    // spg_multiply_to_host: copies of finished row blocks run on their own stream
    cudaStream_t copy_stream = nullptr;
    // page-locked staging for per-product reads of batches (grown on demand)
    void* host_scratch = nullptr;
    size_t host_scratch_bytes = 0;
    // team shape of each numeric bin (0 default, 1 alternative), set by spg_tune
    uint8_t bin_variant[kNumBins] = {};
};

namespace {

constexpr size_t kCtrlBytes = 4096;

struct Failure {
    spg_status status;
    std::string message;
};

spg_status fail(spg_handle* h, spg_status s, const std::string& msg) {
    if (h) h->err = msg;
    return s;
}

void check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    const spg_status s = (e == cudaErrorMemoryAllocation) ? SPG_OUT_OF_MEMORY : SPG_CUDA_ERROR;
    throw Failure{s, std::string(what) + ": " + cudaGetErrorString(e)};
}

// Device allocations of one call; freed on the stream unless released to a result.
class Arena {
public:
    explicit Arena(spg_handle* h) : h_(h) {}
    ~Arena() {
        for (void* p : live_)
            if (p) cudaFreeAsync(p, h_->stream);
    }
    template <typename T>
    T* alloc(size_t count, const char* what) {
        void* p = nullptr;
        check_cuda(cudaMallocAsync(&p, std::max<size_t>(count * sizeof(T), 16), h_->stream), what);
        live_.push_back(p);
        bytes_ += count * sizeof(T);
        return static_cast<T*>(p);
    }
    void release(void* p) {
        for (auto& q : live_)
            if (q == p) q = nullptr;
    }
    void free_now(void* p) {
        for (auto& q : live_)
            if (q == p) {
                cudaFreeAsync(q, h_->stream);
                q = nullptr;
            }
    }
    size_t bytes() const { return bytes_; }

private:
    spg_handle* h_;
    std::vector<void*> live_;
    size_t bytes_ = 0;
};

void sync(spg_handle* h) { check_cuda(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize"); }

// Page-locked host staging of at least `bytes` (control reads go through
// launch_readback into it, never through a copy engine).
void* host_staging(spg_handle* h, size_t bytes) {
    if (bytes > h->host_scratch_bytes) {
        sync(h);
        if (h->host_scratch) cudaFreeHost(h->host_scratch);
        h->host_scratch = nullptr;
        h->host_scratch_bytes = 0;
        const size_t want = std::max<size_t>(bytes, 64 << 10);
        check_cuda(cudaMallocHost(&h->host_scratch, want), "host staging");
        h->host_scratch_bytes = want;
    }
    return h->host_scratch;
}

void require(bool ok, spg_status s, const std::string& msg) {
    if (!ok) throw Failure{s, msg};
}

// Checks what can be checked on the host without reading device memory.
void check_view(const spg_csr_view* m, const char* name) {
    require(m != nullptr, SPG_INVALID_ARGUMENT, std::string(name) + " is NULL");
    require(m->rows >= 0 && m->cols >= 0 && m->nnz >= 0, SPG_INVALID_ARGUMENT,
            std::string(name) + ": negative dimension or nnz");
    require(m->row_ptr != nullptr, SPG_INVALID_ARGUMENT, std::string(name) + ": row_ptr is NULL");
    require(m->nnz == 0 || (m->col && m->val), SPG_INVALID_ARGUMENT, std::string(name) + ": col/val is NULL");
    require(m->location == SPG_HOST || m->location == SPG_DEVICE, SPG_INVALID_ARGUMENT,
            std::string(name) + ": bad location");
    if (m->location == SPG_HOST) {
        require(m->row_ptr[0] == 0 && m->row_ptr[m->rows] == m->nnz, SPG_INVALID_ARGUMENT,
                std::string(name) + ": row_ptr must start at 0 and end at nnz");
    }
}

// A device view of an operand, copying host arrays in.
CsrView stage(spg_handle* h, Arena& ar, const spg_csr_view* m) {
    CsrView v;
    v.rows = m->rows;
    v.cols = m->cols;
    v.nnz = m->nnz;
    if (m->location == SPG_DEVICE) {
        v.rp = m->row_ptr;
        v.ci = m->col;
        v.v = m->val;
        return v;
    }
    int64_t* rp = ar.alloc<int64_t>(static_cast<size_t>(m->rows) + 1, "stage row_ptr");
    int32_t* ci = ar.alloc<int32_t>(static_cast<size_t>(m->nnz), "stage col");
    double* va = ar.alloc<double>(static_cast<size_t>(m->nnz), "stage val");
    check_cuda(cudaMemcpyAsync(rp, m->row_ptr, sizeof(int64_t) * (static_cast<size_t>(m->rows) + 1),
                               cudaMemcpyHostToDevice, h->stream), "H2D row_ptr");
    if (m->nnz) {
        check_cuda(cudaMemcpyAsync(ci, m->col, sizeof(int32_t) * m->nnz, cudaMemcpyHostToDevice, h->stream), "H2D col");
        check_cuda(cudaMemcpyAsync(va, m->val, sizeof(double) * m->nnz, cudaMemcpyHostToDevice, h->stream), "H2D val");
    }
    v.rp = rp;
    v.ci = ci;
    v.v = va;
    return v;
}

struct JobIn {
    const spg_csr_view* A;
    const spg_csr_view* B;
    CsrView S;  // S.rp == nullptr: none
};

struct DevResult {
    int32_t rows = 0, cols = 0;
    int64_t nnz = 0, products = 0;
    int64_t* rp = nullptr;
    int32_t* ci = nullptr;
    double* v = nullptr;
};

struct Ctrl {  // layout of the pinned control block and its device twin
    Stats stats;
    ErrWord err;
    int64_t bin_off[kNumBins + 1];
    unsigned long long cursor[kNumBins];
    int64_t totals[2];  // scanned totals (symbolic, numeric)
};

static_assert(sizeof(Ctrl) % 8 == 0 && sizeof(Ctrl) <= 4096, "Ctrl is read back in 8-byte words into kCtrlBytes");

spg_status map_err(const ErrWord& e, std::string& msg) {
    char buf[160];
    switch (e.code) {
        case kErrColumnRange:
            std::snprintf(buf, sizeof buf, "A contains a column index outside B's row range (A entry %lld)",
                          static_cast<long long>(e.detail));
            msg = buf;
            return SPG_OUT_OF_RANGE_COLUMN;
        case kErrOverflow:
            std::snprintf(buf, sizeof buf, "count overflow (detail %lld)", static_cast<long long>(e.detail));
            msg = buf;
            return SPG_OVERFLOW;
        default:
            std::snprintf(buf, sizeof buf, "malformed CSR input (check %d, detail %lld)", e.where,
                          static_cast<long long>(e.detail));
            msg = buf;
            return SPG_INVALID_ARGUMENT;
    }
}

// The exact (symbolic) mode when asked for, or in auto mode when reserving
// 12 bytes per slot would not fit the budget or half the free memory (slots:
// the scalar products, plus the staged ones of rows above 8192 products).
bool use_exact_mode(spg_handle* h, int64_t products, size_t reserved) {
    if (h->cfg.mode == SPG_MODE_EXACT) return true;
    if (h->cfg.mode == SPG_MODE_UPPER_BOUND) return false;
    const size_t need = static_cast<size_t>(products) * 12;
    if (h->cfg.hbm_budget_bytes && reserved + need > h->cfg.hbm_budget_bytes) return true;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return need > free_b / 2;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// The phase pipeline for one or more products.  Results stay on the device.
// products_out (optional) receives the scalar products of every product.
void run_products(spg_handle* h, const std::vector<JobIn>& in, std::vector<DevResult>& out, bool count_only,
                  int64_t* products_out) {
    cudaStream_t st = h->stream;
    Arena ar(h);
    const int njobs = static_cast<int>(in.size());
    std::vector<Job> jobs(njobs);
    std::vector<int64_t> row_base(njobs + 1, 0);
    for (int j = 0; j < njobs; ++j) {
        check_view(in[j].A, "A");
        check_view(in[j].B, "B");
        require(in[j].A->cols == in[j].B->rows, SPG_INVALID_ARGUMENT, "SpGEMM requires A.cols == B.rows");
        row_base[j + 1] = row_base[j] + in[j].A->rows;
    }
    const int64_t total_rows = row_base[njobs];
    for (int j = 0; j < njobs; ++j) {
        const spg_csr_view* a = in[j].A;
        const spg_csr_view* b = in[j].B;
        jobs[j].A = stage(h, ar, a);
        // C = A*A from one host matrix: copy it to the device once
        const bool same = a->location == b->location && a->row_ptr == b->row_ptr && a->col == b->col &&
                          a->val == b->val && a->rows == b->rows && a->cols == b->cols && a->nnz == b->nnz;
        jobs[j].B = same ? jobs[j].A : stage(h, ar, b);
        jobs[j].S = in[j].S;
        jobs[j].row_base = row_base[j];
    }
    // per-row workspace: ub (rows), cnt and nz (rows + 1 per job)
    const size_t slots = static_cast<size_t>(total_rows + njobs);
    int64_t* ub = ar.alloc<int64_t>(static_cast<size_t>(total_rows), "ub");
    int64_t* cnt = ar.alloc<int64_t>(slots, "cnt");
    int64_t* nz = ar.alloc<int64_t>(slots, "nz");
    int64_t* items = ar.alloc<int64_t>(static_cast<size_t>(total_rows), "items");
    int64_t* d_row_base = ar.alloc<int64_t>(static_cast<size_t>(njobs) + 1, "row_base");
    Ctrl* d_ctrl = ar.alloc<Ctrl>(1, "ctrl");
    Job* d_jobs = ar.alloc<Job>(static_cast<size_t>(njobs), "jobs");
    for (int j = 0; j < njobs; ++j) {
        jobs[j].ub = ub + row_base[j];
        jobs[j].cnt = cnt + row_base[j] + j;
        jobs[j].nz = nz + row_base[j] + j;
    }
    check_cuda(cudaMemsetAsync(cnt, 0, slots * sizeof(int64_t), st), "memset cnt");
    check_cuda(cudaMemsetAsync(nz, 0, slots * sizeof(int64_t), st), "memset nz");
    check_cuda(cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), st), "memset ctrl");
    check_cuda(cudaMemcpyAsync(d_row_base, row_base.data(), sizeof(int64_t) * (njobs + 1), cudaMemcpyHostToDevice, st),
               "H2D row_base");
    check_cuda(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(Job) * njobs, cudaMemcpyHostToDevice, st), "H2D jobs");

    Ctrl* hc = static_cast<Ctrl*>(h->ctrl);
    int64_t launches = total_rows > 0 ? 3 : 1;
    cudaEventRecord(h->ev[0], st);
    launch_rowwork(d_jobs, njobs, d_row_base, total_rows, &d_ctrl->stats, &d_ctrl->err, st);
    launch_bin_offsets(&d_ctrl->stats, d_ctrl->bin_off, st);
    launch_bin_scatter(d_jobs, njobs, d_row_base, total_rows, d_ctrl->bin_off, d_ctrl->cursor, items, st);
    check_cuda(cudaGetLastError(), "K1 launch");
    cudaEventRecord(h->ev[1], st);
    std::vector<int64_t> job_products(njobs, 0);
    int64_t* h_jp = nullptr;
    if (njobs > 1) {
        int64_t* d_jp = ar.alloc<int64_t>(static_cast<size_t>(njobs), "job products");
        h_jp = static_cast<int64_t*>(host_staging(h, sizeof(int64_t) * njobs));
        launch_job_products(d_jobs, njobs, d_row_base, d_jp, st);
        launch_readback(d_jp, h_jp, sizeof(int64_t) * njobs, st);
        launches += 2;
    }
    launch_readback(d_ctrl, hc, sizeof(Ctrl), st);
    ++launches;
    check_cuda(cudaGetLastError(), "readback launch");
    sync(h);  // sync 1: bins and input checks
    if (h_jp) std::copy(h_jp, h_jp + njobs, job_products.begin());
    if (hc->err.code) {
        std::string msg;
        const spg_status s = map_err(hc->err, msg);
        throw Failure{s, msg};
    }
    const int64_t products = static_cast<int64_t>(hc->stats.products);
    const int64_t max_ub = static_cast<int64_t>(hc->stats.max_ub);
    if (njobs == 1) job_products[0] = products;
    if (products_out) std::copy(job_products.begin(), job_products.end(), products_out);
    if (count_only) {
        h->last = spg_timings{};
        h->last.products = products;
        h->last.launches = launches;
        return;
    }
    require(max_ub < (int64_t{1} << 30), SPG_OVERFLOW,
            "an output row has more than 2^30 scalar products (engine limit)");
    int64_t bin_count[kNumBins], bin_off[kNumBins + 1];
    for (int b = 0; b < kNumBins; ++b) bin_count[b] = static_cast<int64_t>(hc->stats.bin_count[b]);
    for (int b = 0; b <= kNumBins; ++b) bin_off[b] = hc->bin_off[b];

    // Output layout: in the upper-bound mode every row is written at the prefix
    // of its product count (ub) and compacted afterwards, and the products of
    // rows above 8192 are also staged (12 more bytes each); in the exact mode a
    // symbolic phase counts the distinct columns of every row first.
    const SplitTotals split = split_totals(hc->stats);
    const bool exact = use_exact_mode(h, products + split.products, ar.bytes());
    size_t scratch_bytes = numeric_scratch_bytes(bin_count, max_ub, split, h->num_sms, !exact);
    if (exact) scratch_bytes = std::max(scratch_bytes, symbolic_scratch_bytes(bin_count, max_ub, h->num_sms));
    void* scratch = scratch_bytes ? ar.alloc<unsigned char>(scratch_bytes, "heavy scratch") : nullptr;
    int64_t* partials = ar.alloc<int64_t>(scan_partials_count(static_cast<int64_t>(slots)), "scan partials");
    // K2 and K4 per bin; in the upper-bound layout the split rows take three
    // K4 launches (planner, pieces, global-slab rows)
    for (int b = 1; b < kNumBins; ++b) launches += bin_count[b] > 0 ? (exact ? 2 : (b > kLastSmemBin ? 3 : 1)) : 0;
    launches += 3;  // scan
    int64_t tmp_total = products;
    // The bins of K2 and K4 run on three streams (warp bins; shared-memory CTA
    // bins; slab and heavy bins, which share the scratch), forked from and
    // joined back into the main stream, so that the tail of one launch overlaps
    // the others.  On one stream (server lanes, the tuner) they run in order.
    const bool one_stream = h->serial_bins || h->one_bin_stream;
    auto stream_of = [&](int b) {
        if (one_stream) return st;
        return b <= kLastWarpBin ? st : (b <= kLastSmemBin ? h->aux[0] : h->aux[1]);
    };
    auto fork = [&] {
        if (one_stream) return;
        cudaEventRecord(h->fork, st);
        for (cudaStream_t a : h->aux) cudaStreamWaitEvent(a, h->fork, 0);
    };
    auto join = [&] {
        if (one_stream) return;
        for (int i = 0; i < 2; ++i) {
            cudaEventRecord(h->join[i], h->aux[i]);
            cudaStreamWaitEvent(st, h->join[i], 0);
        }
    };
    if (exact) {
        fork();
        for (int i = 1; i < kNumBins; ++i) {
            const int b = one_stream ? i : kNumBins - i;
            launch_symbolic(b, d_jobs, items + bin_off[b], bin_count[b], max_ub, scratch, scratch_bytes,
                            &d_ctrl->stats, &d_ctrl->err, stream_of(b), h->num_sms);
        }
        join();
        check_cuda(cudaGetLastError(), "K2 launch");
    }
    cudaEventRecord(h->ev[2], st);
    launch_scan(cnt, static_cast<int64_t>(slots) - 1, partials, st);
    check_cuda(cudaGetLastError(), "K3 launch");
    cudaEventRecord(h->ev[3], st);
    if (exact) {
        launch_readback(cnt + slots - 1, &hc->totals[0], sizeof(int64_t), st);
        launch_readback(&d_ctrl->err, &hc->err, sizeof(ErrWord), st);
        launches += 2;
        sync(h);  // exact mode: size of C
        if (hc->err.code) {
            std::string msg;
            const spg_status s = map_err(hc->err, msg);
            throw Failure{s, msg};
        }
        tmp_total = hc->totals[0];
    }
    if (h->cfg.hbm_budget_bytes && ar.bytes() + static_cast<size_t>(tmp_total) * 12 > h->cfg.hbm_budget_bytes)
        throw Failure{SPG_BUDGET_EXCEEDED, "product footprint exceeds the handle's HBM budget"};
    int32_t* c_col = ar.alloc<int32_t>(static_cast<size_t>(tmp_total), "C col");
    double* c_val = ar.alloc<double>(static_cast<size_t>(tmp_total), "C val");
    for (int j = 0; j < njobs; ++j) {
        jobs[j].c_col = c_col;
        jobs[j].c_val = c_val;
        jobs[j].holes = exact ? 0 : 1;
    }
    check_cuda(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(Job) * njobs, cudaMemcpyHostToDevice, st), "H2D jobs");
    fork();
    // on three streams each stream starts with its largest rows; on one stream the
    // bins go from the smallest rows up (measured faster for overlapping server lanes)
    for (int i = 1; i < kNumBins; ++i) {
        const int b = one_stream ? i : kNumBins - i;
        if (!bin_count[b]) continue;
        cudaStream_t bs = stream_of(b);
        launch_numeric(b, d_jobs, items + bin_off[b], bin_count[b], max_ub, split, scratch, scratch_bytes,
                       &d_ctrl->stats, &d_ctrl->err, bs, h->num_sms, !exact, h->bin_variant[b]);
        cudaEventRecord(h->bin_ev[b], bs);
    }
    join();
    check_cuda(cudaGetLastError(), "K4 launch");
    cudaEventRecord(h->ev[4], st);
    launch_readback(d_ctrl, hc, sizeof(Ctrl), st);
    ++launches;
    sync(h);  // stored count and errors
    if (hc->err.code) {
        std::string msg;
        const spg_status s = map_err(hc->err, msg);
        throw Failure{s, msg};
    }
    const int64_t nz_total = static_cast<int64_t>(hc->stats.nz_total);
    out.resize(njobs);
    if (njobs == 1) {
        int64_t* final_rp = cnt;
        int32_t* final_col = c_col;
        double* final_val = c_val;
        if (nz_total != tmp_total) {  // rows with fewer entries than reserved: compact
            launch_scan(nz, static_cast<int64_t>(slots) - 1, partials, st);
            launches += 4;
            final_col = ar.alloc<int32_t>(static_cast<size_t>(nz_total), "C col (compact)");
            final_val = ar.alloc<double>(static_cast<size_t>(nz_total), "C val (compact)");
            if (exact) launch_compact(d_jobs, in[0].A->rows, final_col, final_val, st);
            else launch_compact_holes(d_jobs, 1, d_row_base, total_rows, final_col, final_val, st);
            check_cuda(cudaGetLastError(), "K5 launch");
            final_rp = nz;
            ar.free_now(c_col);
            ar.free_now(c_val);
        }
        cudaEventRecord(h->ev[5], st);
        DevResult& r = out[0];
        r.rows = in[0].A->rows;
        r.cols = in[0].B->cols;
        r.nnz = nz_total;
        r.rp = final_rp;
        r.ci = final_col;
        r.v = final_val;
        ar.release(final_rp);
        ar.release(final_col);
        ar.release(final_val);
    } else {
        // Every product gets arrays of its own, which the compaction fills
        // directly (row r of product j at its offset minus the product's first
        // offset): the entries of C are moved once, not compacted and then
        // copied out of one flat array.
        launch_scan(nz, static_cast<int64_t>(slots) - 1, partials, st);
        std::vector<int64_t> idx(njobs);
        for (int j = 0; j < njobs; ++j) idx[j] = row_base[j] + j;
        int64_t* d_idx = ar.alloc<int64_t>(static_cast<size_t>(njobs), "start index");
        int64_t* d_starts = ar.alloc<int64_t>(static_cast<size_t>(njobs), "starts");
        check_cuda(cudaMemcpyAsync(d_idx, idx.data(), sizeof(int64_t) * njobs, cudaMemcpyHostToDevice, st),
                   "H2D start index");
        launch_gather(nz, d_idx, d_starts, njobs, st);
        int64_t* h_starts = static_cast<int64_t*>(host_staging(h, sizeof(int64_t) * njobs));
        launch_readback(d_starts, h_starts, sizeof(int64_t) * njobs, st);
        launches += 5;
        sync(h);  // every product's first offset: the sizes of its arrays
        std::vector<int64_t> starts(h_starts, h_starts + njobs);
        starts.push_back(nz_total);
        std::vector<RebaseItem> rb(njobs);
        int64_t max_rows = 0;
        for (int j = 0; j < njobs; ++j) {
            DevResult& r = out[j];
            r.rows = in[j].A->rows;
            r.cols = in[j].B->cols;
            r.nnz = starts[j + 1] - starts[j];
            r.rp = ar.alloc<int64_t>(static_cast<size_t>(r.rows) + 1, "result row_ptr");
            r.ci = ar.alloc<int32_t>(static_cast<size_t>(r.nnz), "result col");
            r.v = ar.alloc<double>(static_cast<size_t>(r.nnz), "result val");
            jobs[j].out_col = r.ci;
            jobs[j].out_val = r.v;
            check_cuda(cudaMemcpyAsync(r.rp, nz + row_base[j] + j, sizeof(int64_t) * (r.rows + 1),
                                       cudaMemcpyDeviceToDevice, st), "D2D row_ptr");
            rb[j] = RebaseItem{r.rp, starts[j], r.rows};
            max_rows = std::max<int64_t>(max_rows, r.rows);
        }
        check_cuda(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(Job) * njobs, cudaMemcpyHostToDevice, st), "H2D jobs");
        if (exact) {
            for (int j = 0; j < njobs; ++j) launch_compact(d_jobs + j, in[j].A->rows, nullptr, nullptr, st);
        } else {
            launch_compact_holes(d_jobs, njobs, d_row_base, total_rows, nullptr, nullptr, st);
        }
        check_cuda(cudaGetLastError(), "K5 launch");
        ar.free_now(c_col);
        ar.free_now(c_val);
        cudaEventRecord(h->ev[5], st);
        RebaseItem* d_rb = ar.alloc<RebaseItem>(static_cast<size_t>(njobs), "rebase items");
        check_cuda(cudaMemcpyAsync(d_rb, rb.data(), sizeof(RebaseItem) * njobs, cudaMemcpyHostToDevice, st),
                   "H2D rebase");
        launch_rebase(d_rb, njobs, max_rows, st);
        check_cuda(cudaGetLastError(), "rebase launch");
        launches += 2 + (exact ? njobs : 1);
        for (auto& r : out) {
            ar.release(r.rp);
            ar.release(r.ci);
            ar.release(r.v);
        }
        sync(h);  // jobs, idx and rb must outlive their copies
    }
    for (int j = 0; j < njobs; ++j) out[j].products = job_products[j];
    sync(h);
    h->last.ms_rowwork = elapsed(h->ev[0], h->ev[1]);
    h->last.ms_symbolic = elapsed(h->ev[1], h->ev[2]);
    h->last.ms_scan = elapsed(h->ev[2], h->ev[3]);
    h->last.ms_numeric = elapsed(h->ev[3], h->ev[4]);
    h->last.ms_compact = elapsed(h->ev[4], h->ev[5]);
    h->last.ms_total = elapsed(h->ev[0], h->ev[5]);
    // per-bin times: launch to launch when the bins ran in sequence (spg_tune),
    // else the time from the fork to the end of each bin
    cudaEvent_t prev = h->ev[3];
    for (int i = 1; i < kNumBins; ++i) {
        const int b = one_stream ? i : kNumBins - i;
        h->last.ms_numeric_bin[b] = 0.0f;
        if (!bin_count[b]) continue;
        h->last.ms_numeric_bin[b] = elapsed(prev, h->bin_ev[b]);
        if (one_stream) prev = h->bin_ev[b];
    }
    h->last.ms_numeric_bin[kBinEmpty] = 0.0f;
    h->last.products = products;
    h->last.nnz = nz_total;
    h->last.rows = total_rows;
    h->last.launches = launches;
    for (int b = 0; b < kNumBins; ++b) h->last.bin_rows[b] = bin_count[b];
}

void free_result_arrays(spg_handle* h, spg_csr_result* c) {
    if (!c) return;
    if (c->location == SPG_DEVICE) {
        if (c->row_ptr) cudaFreeAsync(c->row_ptr, h->stream);
        if (c->col) cudaFreeAsync(c->col, h->stream);
        if (c->val) cudaFreeAsync(c->val, h->stream);
    } else {
        std::free(c->row_ptr);
        std::free(c->col);
        std::free(c->val);
    }
    c->row_ptr = nullptr;
    c->col = nullptr;
    c->val = nullptr;
    c->nnz = 0;
}

// Converts a device result into the caller's requested location.
void deliver(spg_handle* h, DevResult& r, int32_t loc, spg_csr_result* C) {
    std::memset(C, 0, sizeof(*C));
    C->rows = r.rows;
    C->cols = r.cols;
    C->nnz = r.nnz;
    C->products = r.products;
    if (loc == SPG_DEVICE) {
        C->location = SPG_DEVICE;
        C->row_ptr = r.rp;
        C->col = r.ci;
        C->val = r.v;
        return;
    }
    C->location = SPG_HOST;
    C->row_ptr = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (static_cast<size_t>(r.rows) + 1)));
    C->col = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max<int64_t>(r.nnz, 1)));
    C->val = static_cast<double*>(std::malloc(sizeof(double) * std::max<int64_t>(r.nnz, 1)));
    cudaError_t e = cudaSuccess;
    if (!C->row_ptr || !C->col || !C->val) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(C->row_ptr, r.rp, sizeof(int64_t) * (static_cast<size_t>(r.rows) + 1),
                            cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && r.nnz)
        e = cudaMemcpyAsync(C->col, r.ci, sizeof(int32_t) * r.nnz, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && r.nnz)
        e = cudaMemcpyAsync(C->val, r.v, sizeof(double) * r.nnz, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFreeAsync(r.rp, h->stream);
    cudaFreeAsync(r.ci, h->stream);
    cudaFreeAsync(r.v, h->stream);
    if (e != cudaSuccess) {
        free_result_arrays(h, C);
        check_cuda(e, "D2H result");
    }
}

template <typename F>
spg_status guarded(spg_handle* h, F&& body) {
    if (!h) return SPG_INVALID_ARGUMENT;
    cudaSetDevice(h->device);
    try {
        body();
        h->err.clear();
        return SPG_OK;
    } catch (const Failure& f) {
        return fail(h, f.status, f.message);
    } catch (const std::bad_alloc&) {
        return fail(h, SPG_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(h, SPG_CUDA_ERROR, e.what());
    }
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

spg_status spg_config_default(spg_config* c) {
    if (!c) return SPG_INVALID_ARGUMENT;
    std::memset(c, 0, sizeof(*c));
    return SPG_OK;
}

spg_status spg_create(const spg_config* config, spg_handle** out) {
    if (!out) return SPG_INVALID_ARGUMENT;
    *out = nullptr;
    spg_config cfg;
    spg_config_default(&cfg);
    if (config) cfg = *config;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return SPG_CUDA_ERROR;
    }
    if (cfg.device < 0 || cfg.device >= ndev) return SPG_INVALID_ARGUMENT;
    if (cfg.bin_streams != 0 && cfg.bin_streams != 1 && cfg.bin_streams != 3) return SPG_INVALID_ARGUMENT;
    auto* h = new spg_handle;
    h->cfg = cfg;
    h->device = cfg.device;
    h->one_bin_stream = cfg.bin_streams == 1;
    if (cudaSetDevice(h->device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&h->ctrl, kCtrlBytes) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return SPG_CUDA_ERROR;
    }
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
    for (auto& e : h->ev) cudaEventCreate(&e);
    for (auto& e : h->bin_ev) cudaEventCreate(&e);
    for (auto& a : h->aux) cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming);
    for (auto& e : h->join) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, h->device) == cudaSuccess) {
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
    *out = h;
    return SPG_OK;
}

void spg_destroy(spg_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->acc_has) free_result_arrays(h, &h->acc);
    cudaStreamSynchronize(h->stream);
    if (h->copy_stream) {
        cudaStreamSynchronize(h->copy_stream);
        cudaStreamDestroy(h->copy_stream);
    }
    if (h->host_scratch) cudaFreeHost(h->host_scratch);
    for (auto& e : h->ev) cudaEventDestroy(e);
    for (auto& e : h->bin_ev) cudaEventDestroy(e);
    for (auto a : h->aux) {
        cudaStreamSynchronize(a);
        cudaStreamDestroy(a);
    }
    cudaEventDestroy(h->fork);
    for (auto e : h->join) cudaEventDestroy(e);
    cudaStreamDestroy(h->stream);
    cudaFreeHost(h->ctrl);
    delete h;
}

const char* spg_last_error(const spg_handle* h) { return h ? h->err.c_str() : "NULL handle"; }

const char* spg_status_string(spg_status s) {
    switch (s) {
        case SPG_OK: return "SPG_OK";
        case SPG_INVALID_ARGUMENT: return "SPG_INVALID_ARGUMENT";
        case SPG_OVERFLOW: return "SPG_OVERFLOW";
        case SPG_OUT_OF_RANGE_COLUMN: return "SPG_OUT_OF_RANGE_COLUMN";
        case SPG_OUT_OF_MEMORY: return "SPG_OUT_OF_MEMORY";
        case SPG_BUDGET_EXCEEDED: return "SPG_BUDGET_EXCEEDED";
        case SPG_DEVICE_TIMEOUT: return "SPG_DEVICE_TIMEOUT";
        case SPG_CUDA_ERROR: return "SPG_CUDA_ERROR";
        case SPG_NOT_READY: return "SPG_NOT_READY";
        case SPG_CANCELLED: return "SPG_CANCELLED";
        case SPG_FORMAT_ERROR: return "SPG_FORMAT_ERROR";
    }
    return "unknown spg_status";
}

void* spg_stream(spg_handle* h) { return h ? static_cast<void*>(h->stream) : nullptr; }

spg_status spg_multiply(spg_handle* h, const spg_csr_view* A, const spg_csr_view* B, int32_t out_location,
                        spg_csr_result* C) {
    return guarded(h, [&] {
        require(C != nullptr, SPG_INVALID_ARGUMENT, "C is NULL");
        require(out_location == SPG_HOST || out_location == SPG_DEVICE, SPG_INVALID_ARGUMENT, "bad out_location");
        std::vector<JobIn> in{{A, B, CsrView{}}};
        std::vector<DevResult> out;
        run_products(h, in, out, false, nullptr);
        deliver(h, out[0], out_location, C);
    });
}

// Operands with at least this many entries in A are multiplied in row blocks.
constexpr int64_t kBlockedEntries = int64_t{1} << 22;

spg_status spg_multiply_to_host(spg_handle* h, const spg_csr_view* A, const spg_csr_view* B, int64_t* c_row_ptr,
                                int32_t* c_col, double* c_val, int64_t c_capacity, int64_t* c_nnz) {
    return guarded(h, [&] {
        require(A && B && c_row_ptr && c_nnz && c_capacity >= 0 && (c_capacity == 0 || (c_col && c_val)),
                SPG_INVALID_ARGUMENT, "bad spg_multiply_to_host arguments");
        check_view(A, "A");
        check_view(B, "B");
        require(A->cols == B->rows, SPG_INVALID_ARGUMENT, "SpGEMM requires A.cols == B.rows");
        *c_nnz = 0;
        if (!h->copy_stream)
            check_cuda(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking), "copy stream");
        cudaStream_t st = h->stream, cs = h->copy_stream;
        // operands on the device once for all row blocks
        Arena ar(h);
        const spg_csr_view* views[2] = {A, B};
        spg_csr_view dv[2];
        for (int i = 0; i < 2; ++i) {
            dv[i] = *views[i];
            if (views[i]->location == SPG_HOST) {
                const bool same = i == 1 && B->row_ptr == A->row_ptr && B->col == A->col && B->val == A->val &&
                                  B->rows == A->rows && B->cols == A->cols && B->nnz == A->nnz;
                const CsrView v = same ? CsrView{} : stage(h, ar, views[i]);
                if (same) dv[1] = dv[0];
                else {
                    dv[i].row_ptr = v.rp;
                    dv[i].col = v.ci;
                    dv[i].val = v.v;
                    dv[i].location = SPG_DEVICE;
                }
            }
        }
        // Row blocks by A's entries: 1/32, 1/32, 1/16, then 1/8 each, so that the first
        // copy starts after a small block and the later blocks keep the copy engine
        // busy while the next one computes.  Small operands run as one block.  The
        // cuts come from A's row offsets on the host, or from equal row counts
        // when A lives on the device.
        const int32_t m = A->rows;
        std::vector<int32_t> cut{0};
        if (A->nnz >= kBlockedEntries && m > 1) {
            const double fr[] = {1.0 / 32, 1.0 / 32, 1.0 / 16, 1.0 / 8, 1.0 / 8, 1.0 / 8, 1.0 / 8,
                                 1.0 / 8, 1.0 / 8, 1.0 / 8};
            double acc = 0.0;
            for (double f : fr) {
                acc += f;
                int32_t r;
                if (acc >= 1.0 - 1e-12) {
                    r = m;
                } else if (A->location == SPG_HOST) {
                    const int64_t target = static_cast<int64_t>(acc * static_cast<double>(A->nnz));
                    r = static_cast<int32_t>(std::lower_bound(A->row_ptr, A->row_ptr + m + 1, target) - A->row_ptr);
                } else {
                    r = static_cast<int32_t>(acc * m);
                }
                r = std::min(std::max(r, cut.back()), m);
                if (r > cut.back()) cut.push_back(r);
            }
        }
        if (cut.back() != m) cut.push_back(m);
        const int nchunks = static_cast<int>(cut.size()) - 1;
        int64_t products = 0;
        spg_timings sum{};
        int64_t off = 0;
        std::vector<cudaEvent_t> done;
        // Block results stay allocated until every copy has finished: memory freed
        // on the copy stream and reused by the compute stream would make the
        // compute wait for the copies (the pool orders reuse after the free).
        std::vector<DevResult> held;
        auto release_held = [&] {
            for (auto& q : held) {
                cudaFreeAsync(q.rp, st);
                cudaFreeAsync(q.ci, st);
                cudaFreeAsync(q.v, st);
            }
            held.clear();
        };
        // On any failure after the first block (a capacity shortfall, an input
        // error found in a later block, a CUDA error), copies of earlier blocks
        // into the caller's host arrays may still be queued on the copy stream:
        // wait for them before returning, so that the caller can free or reuse
        // its buffers, and release the blocks and events.
        auto abandon = [&] {
            cudaStreamSynchronize(cs);
            release_held();
            for (auto e : done) cudaEventDestroy(e);
            done.clear();
        };
        c_row_ptr[0] = 0;
        try {
            for (int k = 0; k < nchunks; ++k) {
                const int32_t r0 = cut[k], r1 = cut[k + 1];
                spg_csr_view blk = dv[0];
                blk.rows = r1 - r0;
                blk.row_ptr = dv[0].row_ptr + r0;  // absolute offsets into A's column/value arrays
                std::vector<JobIn> in{{&blk, &dv[1], CsrView{}}};
                std::vector<DevResult> out;
                run_products(h, in, out, false, nullptr);
                DevResult& r = out[0];
                held.push_back(r);  // freed by release_held, on success or failure
                if (off + r.nnz > c_capacity) {
                    *c_nnz = off + r.nnz;  // at least this many entries are needed
                    throw Failure{SPG_BUDGET_EXCEEDED, "nnz(C) exceeds c_capacity"};
                }
                // this block's offsets continue the previous ones; copy it out on the copy stream
                launch_add_offset(r.rp + 1, r.rows, off, st);
                cudaEvent_t e;
                check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
                done.push_back(e);
                check_cuda(cudaEventRecord(e, st), "event record");
                check_cuda(cudaStreamWaitEvent(cs, e, 0), "stream wait");
                check_cuda(cudaMemcpyAsync(c_row_ptr + r0 + 1, r.rp + 1, sizeof(int64_t) * r.rows, cudaMemcpyDeviceToHost, cs),
                           "D2H row_ptr");
                if (r.nnz) {
                    check_cuda(cudaMemcpyAsync(c_col + off, r.ci, sizeof(int32_t) * r.nnz, cudaMemcpyDeviceToHost, cs),
                               "D2H col");
                    check_cuda(cudaMemcpyAsync(c_val + off, r.v, sizeof(double) * r.nnz, cudaMemcpyDeviceToHost, cs),
                               "D2H val");
                }
                off += r.nnz;
                sum.ms_rowwork += h->last.ms_rowwork;
                sum.ms_symbolic += h->last.ms_symbolic;
                sum.ms_scan += h->last.ms_scan;
                sum.ms_numeric += h->last.ms_numeric;
                sum.ms_compact += h->last.ms_compact;
                sum.ms_total += h->last.ms_total;
                sum.launches += h->last.launches + 1;
                products += r.products;
                for (int b = 0; b < kNumBins; ++b) {
                    sum.bin_rows[b] += h->last.bin_rows[b];
                    sum.ms_numeric_bin[b] += h->last.ms_numeric_bin[b];
                }
            }
        } catch (...) {
            abandon();
            throw;
        }
        check_cuda(cudaStreamSynchronize(cs), "copy stream");
        release_held();
        for (auto e : done) cudaEventDestroy(e);
        *c_nnz = off;
        sum.products = products;
        sum.nnz = off;
        sum.rows = m;
        h->last = sum;
    });
}

spg_status spg_result_download(spg_handle* h, const spg_csr_result* C, int64_t* row_ptr, int32_t* col, double* val) {
    return guarded(h, [&] {
        require(C != nullptr && C->location == SPG_DEVICE, SPG_INVALID_ARGUMENT, "not a device result");
        if (row_ptr)
            check_cuda(cudaMemcpyAsync(row_ptr, C->row_ptr, sizeof(int64_t) * (static_cast<size_t>(C->rows) + 1),
                                       cudaMemcpyDeviceToHost, h->stream), "D2H row_ptr");
        if (col && C->nnz)
            check_cuda(cudaMemcpyAsync(col, C->col, sizeof(int32_t) * C->nnz, cudaMemcpyDeviceToHost, h->stream),
                       "D2H col");
        if (val && C->nnz)
            check_cuda(cudaMemcpyAsync(val, C->val, sizeof(double) * C->nnz, cudaMemcpyDeviceToHost, h->stream),
                       "D2H val");
        sync(h);
    });
}

spg_status spg_result_free(spg_handle* h, spg_csr_result* C) {
    return guarded(h, [&] { free_result_arrays(h, C); });
}

spg_status spg_scalar_multiplication_count(spg_handle* h, const spg_csr_view* A, const spg_csr_view* B,
                                           int64_t* products) {
    return guarded(h, [&] {
        require(products != nullptr, SPG_INVALID_ARGUMENT, "products is NULL");
        std::vector<JobIn> in{{A, B, CsrView{}}};
        std::vector<DevResult> out;
        run_products(h, in, out, true, products);
    });
}

spg_status spg_partition_rows(spg_handle* h, const spg_csr_view* A, const spg_csr_view* B, int32_t parts,
                              int32_t* first_row) {
    return guarded(h, [&] {
        require(parts >= 1 && first_row != nullptr, SPG_INVALID_ARGUMENT, "parts must be >= 1, first_row non-NULL");
        check_view(A, "A");
        check_view(B, "B");
        require(A->cols == B->rows, SPG_INVALID_ARGUMENT, "SpGEMM requires A.cols == B.rows");
        cudaStream_t st = h->stream;
        Arena ar(h);
        Job job;
        job.A = stage(h, ar, A);
        const bool same = A->location == B->location && A->row_ptr == B->row_ptr && A->col == B->col &&
                          A->val == B->val && A->rows == B->rows && A->cols == B->cols && A->nnz == B->nnz;
        job.B = same ? job.A : stage(h, ar, B);
        const int64_t m = A->rows;
        int64_t* ub = ar.alloc<int64_t>(static_cast<size_t>(m) + 1, "row products");
        int64_t* cnt = ar.alloc<int64_t>(static_cast<size_t>(m) + 1, "row reservation");
        job.ub = ub;
        job.cnt = cnt;
        int64_t* d_row_base = ar.alloc<int64_t>(2, "row base");
        Ctrl* d_ctrl = ar.alloc<Ctrl>(1, "ctrl");
        Job* d_job = ar.alloc<Job>(1, "job");
        const size_t first_words = (static_cast<size_t>(parts) + 2) / 2;  // parts + 1 int32, read in 8-byte words
        int32_t* d_first = ar.alloc<int32_t>(2 * first_words, "first rows");
        int64_t* partials = ar.alloc<int64_t>(scan_partials_count(m + 1), "scan partials");
        const int64_t rb[2] = {0, m};
        check_cuda(cudaMemsetAsync(ub, 0, sizeof(int64_t) * (static_cast<size_t>(m) + 1), st), "memset");
        check_cuda(cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), st), "memset ctrl");
        check_cuda(cudaMemcpyAsync(d_row_base, rb, sizeof rb, cudaMemcpyHostToDevice, st), "H2D row base");
        check_cuda(cudaMemcpyAsync(d_job, &job, sizeof job, cudaMemcpyHostToDevice, st), "H2D job");
        launch_rowwork(d_job, 1, d_row_base, m, &d_ctrl->stats, &d_ctrl->err, st);
        launch_scan(ub, m, partials, st);  // exclusive, ub[m] = all scalar products
        launch_partition(ub, m, parts, d_first, st);
        check_cuda(cudaGetLastError(), "partition launch");
        Ctrl* hc = static_cast<Ctrl*>(h->ctrl);
        void* hf = host_staging(h, 8 * first_words);
        launch_readback(&d_ctrl->err, &hc->err, sizeof(ErrWord), st);
        launch_readback(d_first, hf, 8 * first_words, st);
        sync(h);  // rb and job must outlive their copies
        if (hc->err.code) {
            std::string msg;
            const spg_status status = map_err(hc->err, msg);
            throw Failure{status, msg};
        }
        std::memcpy(first_row, hf, sizeof(int32_t) * (static_cast<size_t>(parts) + 1));
    });
}

spg_status spg_scalar_multiplication_count_batch(spg_handle* h, int32_t n, const spg_csr_view* A,
                                                 const spg_csr_view* B, int64_t* products) {
    return guarded(h, [&] {
        require(n >= 0 && (n == 0 || (A && B && products)), SPG_INVALID_ARGUMENT, "bad batch arguments");
        if (n == 0) return;
        std::vector<JobIn> in(n);
        for (int i = 0; i < n; ++i) in[i] = {&A[i], &B[i], CsrView{}};
        std::vector<DevResult> out;
        run_products(h, in, out, true, products);
    });
}

spg_status spg_tune(spg_handle* h, const spg_csr_view* A, const spg_csr_view* B, int32_t reps,
                    spg_tune_report* report) {
    return guarded(h, [&] {
        require(reps >= 1 && reps <= 64, SPG_INVALID_ARGUMENT, "reps must be in [1, 64]");
        uint8_t saved[kNumBins];
        std::memcpy(saved, h->bin_variant, sizeof saved);
        spg_tune_report rep{};
        struct SerialBins {  // per-bin times need the bins one after the other
            spg_handle* h;
            explicit SerialBins(spg_handle* x) : h(x) { h->serial_bins = true; }
            ~SerialBins() { h->serial_bins = false; }
        } serial(h);
        try {
            std::vector<JobIn> in{{A, B, CsrView{}}};
            auto one_call = [&] {
                std::vector<DevResult> out;
                run_products(h, in, out, false, nullptr);
                for (auto& o : out) {
                    cudaFreeAsync(o.rp, h->stream);
                    cudaFreeAsync(o.ci, h->stream);
                    cudaFreeAsync(o.v, h->stream);
                }
            };
            for (int v = 0; v < kNumVariants; ++v) {
                std::memset(h->bin_variant, v, sizeof h->bin_variant);
                std::vector<std::vector<float>> t(kNumBins);
                for (int r = 0; r <= reps; ++r) {  // the first run warms up
                    one_call();
                    if (r == 0) continue;
                    for (int b = 0; b < kNumBins; ++b) t[b].push_back(h->last.ms_numeric_bin[b]);
                }
                for (int b = 0; b < kNumBins; ++b) {
                    std::sort(t[b].begin(), t[b].end());
                    rep.ms_bin[v][b] = t[b][t[b].size() / 2];
                }
                for (int b = 0; b < kNumBins; ++b) rep.bin_rows[b] = h->last.bin_rows[b];
                rep.products = h->last.products;
            }
            for (int b = 0; b < kNumBins; ++b)  // candidates: the alternative measurably faster alone
                rep.variant[b] = (rep.bin_rows[b] > 0 && rep.ms_bin[1][b] < 0.97f * rep.ms_bin[0][b]) ? 1 : 0;
            // Each candidate is then confirmed as calls run (the bins on their
            // streams, beside one another): a bin alone can time differently
            // from the same bin sharing the GPU with the other bins (on the
            // power-law product, one alternative 3% faster alone made the whole
            // numeric phase 1.7% slower).  A candidate stays only where the
            // median numeric phase with it is at least 0.5% shorter than without.
            h->serial_bins = false;
            auto numeric_ms = [&](const uint8_t* variants) {
                std::memcpy(h->bin_variant, variants, sizeof h->bin_variant);
                std::vector<float> t;
                for (int r = 0; r <= reps; ++r) {
                    one_call();
                    if (r > 0) t.push_back(h->last.ms_numeric);
                }
                std::sort(t.begin(), t.end());
                return t[t.size() / 2];
            };
            if (!h->one_bin_stream)
                for (int b = 0; b < kNumBins; ++b) {
                    if (!rep.variant[b]) continue;
                    uint8_t without[kNumBins];
                    std::memcpy(without, rep.variant, sizeof without);
                    without[b] = 0;
                    const float ms_with = numeric_ms(rep.variant);
                    const float ms_without = numeric_ms(without);
                    if (!(ms_with < 0.995f * ms_without)) rep.variant[b] = 0;
                }
        } catch (...) {
            std::memcpy(h->bin_variant, saved, sizeof saved);
            throw;
        }
        std::memcpy(h->bin_variant, rep.variant, sizeof h->bin_variant);
        if (report) *report = rep;
    });
}

spg_status spg_validate_full(spg_handle* h, const spg_csr_view* A, const spg_csr_view* B, const spg_csr_view* C,
                             spg_full_report* rep) {
    return guarded(h, [&] {
        require(A && B && C && rep, SPG_INVALID_ARGUMENT, "bad validation arguments");
        check_view(A, "A");
        check_view(B, "B");
        check_view(C, "C");
        std::memset(rep, 0, sizeof(*rep));
        rep->environment_ok = 1;  // IEEE FP64, round to nearest, gradual underflow on the device
        rep->max_abs_error = std::numeric_limits<double>::infinity();
        rep->rejected = 1;
        cudaStream_t st = h->stream;
        Arena ar(h);
        const CsrView a = stage(h, ar, A);
        const CsrView b = stage(h, ar, B);
        const CsrView c = stage(h, ar, C);
        int* d_flag = ar.alloc<int>(1, "flag");
        check_cuda(cudaMemsetAsync(d_flag, 0, sizeof(int), st), "memset");
        const bool shapes = A->cols == B->rows && C->rows == A->rows && C->cols == B->cols;
        launch_validate_csr(a, false, d_flag, st);
        launch_validate_csr(b, false, d_flag, st);
        launch_validate_csr(c, true, d_flag, st);
        int* h_flag = static_cast<int*>(host_staging(h, 64));
        launch_readback(d_flag, h_flag, 8, st);  // flag plus padding (allocations are >= 16 bytes)
        sync(h);
        rep->matrices_ok = shapes && h_flag[0] == 0;
        if (!rep->matrices_ok) return;
        const int32_t m = A->rows;
        int64_t* slot_off = ar.alloc<int64_t>(static_cast<size_t>(m) + 1, "slots");
        int64_t* partials = ar.alloc<int64_t>(scan_partials_count(static_cast<int64_t>(m) + 1), "partials");
        check_cuda(cudaMemsetAsync(slot_off, 0, sizeof(int64_t) * (static_cast<size_t>(m) + 1), st), "memset");
        launch_validate_slots(a, b, slot_off, st);
        launch_scan(slot_off, m, partials, st);
        std::vector<int64_t> off(static_cast<size_t>(m) + 1);
        int64_t* h_off = static_cast<int64_t*>(host_staging(h, sizeof(int64_t) * (static_cast<size_t>(m) + 1)));
        launch_readback(slot_off, h_off, sizeof(int64_t) * (static_cast<size_t>(m) + 1), st);
        const int nb = validate_hist_buckets();
        unsigned long long* d_counters = ar.alloc<unsigned long long>(8, "counters");
        double* d_maxima = ar.alloc<double>(4, "maxima");
        unsigned long long* d_hist = ar.alloc<unsigned long long>(static_cast<size_t>(nb), "histogram");
        check_cuda(cudaMemsetAsync(d_counters, 0, 8 * sizeof(unsigned long long), st), "memset");
        check_cuda(cudaMemsetAsync(d_maxima, 0, 4 * sizeof(double), st), "memset");
        check_cuda(cudaMemsetAsync(d_hist, 0, sizeof(unsigned long long) * nb, st), "memset");
        sync(h);
        std::copy(h_off, h_off + m + 1, off.begin());
        // row chunks whose tables fit kChunkCells cells (a bigger row alone gets its own)
        constexpr int64_t kChunkCells = int64_t{1} << 27;
        int64_t max_chunk = 0;
        std::vector<int32_t> cuts{0};
        for (int32_t r = 0; r < m;) {
            int32_t e = r + 1;
            while (e < m && off[e + 1] - off[r] <= kChunkCells) ++e;
            max_chunk = std::max(max_chunk, off[e] - off[r]);
            cuts.push_back(e);
            r = e;
        }
        void* table = ar.alloc<unsigned char>(static_cast<size_t>(max_chunk) * validate_cell_bytes(), "cell tables");
        for (size_t i = 0; i + 1 < cuts.size(); ++i)
            launch_validate_rows(a, b, c, cuts[i], cuts[i + 1], slot_off, table, d_counters, d_maxima, d_hist, st);
        check_cuda(cudaGetLastError(), "validation launch");
        const size_t back = 8 * sizeof(unsigned long long) + 4 * sizeof(double) + sizeof(unsigned long long) * nb;
        unsigned char* hb = static_cast<unsigned char*>(host_staging(h, back));
        launch_readback(d_counters, hb, 8 * sizeof(unsigned long long), st);
        launch_readback(d_maxima, hb + 64, 4 * sizeof(double), st);
        launch_readback(d_hist, hb + 96, sizeof(unsigned long long) * nb, st);
        sync(h);
        const unsigned long long* cnt = reinterpret_cast<const unsigned long long*>(hb);
        const double* mx = reinterpret_cast<const double*>(hb + 64);
        const unsigned long long* hist = reinterpret_cast<const unsigned long long*>(hb + 96);
        rep->rejected = static_cast<int64_t>(cnt[0]);
        rep->row_nnz_mismatches = static_cast<int64_t>(cnt[1]);
        rep->support_mismatches = static_cast<int64_t>(cnt[2]);
        rep->reference_nnz = static_cast<int64_t>(cnt[3]);
        rep->checked_coordinates = static_cast<int64_t>(cnt[4]);
        rep->max_abs_error = mx[0];
        rep->max_error_ratio = mx[1];
        rep->max_rel_error = mx[2];
        unsigned long long total = 0;
        for (int i = 0; i < nb; ++i) total += hist[i];
        if (total) {
            unsigned long long seen = 0;
            int i = 0;
            for (; i < nb; ++i) {
                seen += hist[i];
                if (seen > total / 2) break;
            }
            // bucket i holds the doubles whose top 14 bits are i: report its midpoint
            uint64_t lo_bits = static_cast<uint64_t>(i) << 49, hi_bits = (static_cast<uint64_t>(i) + 1) << 49;
            double lo, hi;
            std::memcpy(&lo, &lo_bits, 8);
            std::memcpy(&hi, &hi_bits, 8);
            rep->median_rel_error = 0.5 * (lo + hi);
        }
        rep->passed = rep->rejected == 0;
        rep->partial_passed = rep->row_nnz_mismatches == 0;
    });
}

spg_status spg_transpose(spg_handle* h, const spg_csr_view* A, int32_t out_location, spg_csr_result* C) {
    return guarded(h, [&] {
        require(C != nullptr, SPG_INVALID_ARGUMENT, "C is NULL");
        require(out_location == SPG_HOST || out_location == SPG_DEVICE, SPG_INVALID_ARGUMENT, "bad out_location");
        check_view(A, "A");
        cudaStream_t st = h->stream;
        Arena ar(h);
        const CsrView a = stage(h, ar, A);
        int* d_flag = ar.alloc<int>(1, "flag");
        check_cuda(cudaMemsetAsync(d_flag, 0, sizeof(int), st), "memset");
        launch_validate_csr(a, false, d_flag, st, false);
        int* h_flag = static_cast<int*>(host_staging(h, 64));
        launch_readback(d_flag, h_flag, 8, st);
        sync(h);
        require(h_flag[0] == 0, SPG_INVALID_ARGUMENT, "malformed CSR operand (offsets or columns out of range)");
        DevResult r;
        r.rows = A->cols;
        r.cols = A->rows;
        r.nnz = A->nnz;
        r.rp = ar.alloc<int64_t>(static_cast<size_t>(A->cols) + 1, "transpose row_ptr");
        r.ci = ar.alloc<int32_t>(static_cast<size_t>(A->nnz), "transpose col");
        r.v = ar.alloc<double>(static_cast<size_t>(A->nnz), "transpose val");
        void* scratch = ar.alloc<unsigned char>(transpose_scratch_bytes(A->nnz, A->cols), "transpose scratch");
        launch_transpose(a.rp, a.ci, a.v, A->rows, A->cols, A->nnz, r.rp, r.ci, r.v, scratch, st);
        check_cuda(cudaGetLastError(), "transpose launch");
        ar.release(r.rp);
        ar.release(r.ci);
        ar.release(r.v);
        deliver(h, r, out_location, C);
    });
}

spg_status spg_get_bin_variants(const spg_handle* h, uint8_t* variants) {
    if (!h || !variants) return SPG_INVALID_ARGUMENT;
    std::memcpy(variants, h->bin_variant, kNumBins);
    return SPG_OK;
}

spg_status spg_set_bin_variants(spg_handle* h, const uint8_t* variants) {
    if (!h || !variants) return SPG_INVALID_ARGUMENT;
    for (int b = 0; b < kNumBins; ++b)
        if (variants[b] >= kNumVariants) return SPG_INVALID_ARGUMENT;
    std::memcpy(h->bin_variant, variants, kNumBins);
    return SPG_OK;
}

spg_status spg_last_timings(const spg_handle* h, spg_timings* t) {
    if (!h || !t) return SPG_INVALID_ARGUMENT;
    *t = h->last;
    return SPG_OK;
}

spg_status spg_accum_begin(spg_handle* h, int32_t rows, int32_t cols) {
    return guarded(h, [&] {
        require(rows >= 0 && cols >= 0, SPG_INVALID_ARGUMENT, "negative accumulator shape");
        if (h->acc_has) free_result_arrays(h, &h->acc);
        h->acc_has = false;
        h->acc_active = true;
        h->acc_rows = rows;
        h->acc_cols = cols;
    });
}

spg_status spg_accum_add(spg_handle* h, const spg_csr_view* A, const spg_csr_view* B) {
    return guarded(h, [&] {
        require(h->acc_active, SPG_INVALID_ARGUMENT, "no accumulation in progress");
        require(A && B, SPG_INVALID_ARGUMENT, "A or B is NULL");
        require(A->cols == B->rows && A->rows == h->acc_rows && B->cols == h->acc_cols, SPG_INVALID_ARGUMENT,
                "incompatible Trident partial product shapes");
        CsrView S;
        if (h->acc_has) {
            S.rows = h->acc.rows;
            S.cols = h->acc.cols;
            S.nnz = h->acc.nnz;
            S.rp = h->acc.row_ptr;
            S.ci = h->acc.col;
            S.v = h->acc.val;
        }
        std::vector<JobIn> in{{A, B, S}};
        std::vector<DevResult> out;
        run_products(h, in, out, false, nullptr);
        if (h->acc_has) free_result_arrays(h, &h->acc);
        deliver(h, out[0], SPG_DEVICE, &h->acc);
        h->acc_has = true;
    });
}

// Like the reference's `CsrMatrix finish() const`, this returns a copy of the
// current sum and leaves the accumulation as it is (more stages may follow).
spg_status spg_accum_finish(spg_handle* h, int32_t out_location, spg_csr_result* C) {
    return guarded(h, [&] {
        require(h->acc_active, SPG_INVALID_ARGUMENT, "no accumulation in progress");
        require(C != nullptr, SPG_INVALID_ARGUMENT, "C is NULL");
        require(out_location == SPG_HOST || out_location == SPG_DEVICE, SPG_INVALID_ARGUMENT, "bad out_location");
        DevResult r;
        r.rows = h->acc_rows;
        r.cols = h->acc_cols;
        r.nnz = h->acc_has ? h->acc.nnz : 0;
        r.products = h->acc_has ? h->acc.products : 0;
        const size_t rp_bytes = sizeof(int64_t) * (static_cast<size_t>(r.rows) + 1);
        check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&r.rp), rp_bytes, h->stream), "alloc row_ptr");
        check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&r.ci), std::max<size_t>(16, 4 * r.nnz), h->stream),
                   "alloc col");
        check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&r.v), std::max<size_t>(16, 8 * r.nnz), h->stream),
                   "alloc val");
        if (h->acc_has) {
            check_cuda(cudaMemcpyAsync(r.rp, h->acc.row_ptr, rp_bytes, cudaMemcpyDeviceToDevice, h->stream), "D2D");
            if (r.nnz) {
                check_cuda(cudaMemcpyAsync(r.ci, h->acc.col, 4 * r.nnz, cudaMemcpyDeviceToDevice, h->stream), "D2D");
                check_cuda(cudaMemcpyAsync(r.v, h->acc.val, 8 * r.nnz, cudaMemcpyDeviceToDevice, h->stream), "D2D");
            }
        } else {  // no stage added yet: an all-empty result
            check_cuda(cudaMemsetAsync(r.rp, 0, rp_bytes, h->stream), "memset");
        }
        deliver(h, r, out_location, C);
    });
}

spg_status spg_accum_end(spg_handle* h) {
    return guarded(h, [&] {
        if (h->acc_has) free_result_arrays(h, &h->acc);
        h->acc_has = false;
        h->acc_active = false;
    });
}

spg_status spg_multiply_batch(spg_handle* h, int32_t n, const spg_csr_view* A, const spg_csr_view* B,
                              int32_t out_location, spg_csr_result* C) {
    return guarded(h, [&] {
        require(n >= 0 && (n == 0 || (A && B && C)), SPG_INVALID_ARGUMENT, "bad batch arguments");
        require(out_location == SPG_HOST || out_location == SPG_DEVICE, SPG_INVALID_ARGUMENT, "bad out_location");
        if (n == 0) return;
        std::vector<JobIn> in(n);
        for (int i = 0; i < n; ++i) in[i] = {&A[i], &B[i], CsrView{}};
        std::vector<DevResult> out;
        run_products(h, in, out, false, nullptr);
        for (int i = 0; i < n; ++i) deliver(h, out[i], out_location, &C[i]);
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Plans: the structure-dependent phases once, the value-dependent phases as a
// CUDA graph replayed by spg_plan_execute.
struct spg_plan {
    spg_handle* h = nullptr;
    int njobs = 0;
    std::vector<int64_t> row_base;     // njobs + 1
    std::vector<int32_t> rows, cols;
    std::vector<int64_t> job_products;
    std::vector<void*> bufs;           // device allocations owned by the plan
    int64_t* rp = nullptr;             // per-product offsets (rebased), slots entries
    int32_t* col = nullptr;
    double* val = nullptr;
    Ctrl* hc = nullptr;                // page-locked readbacks
    int64_t* h_starts = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool executed = false;
    int64_t nz_total = 0;
    std::vector<int64_t> starts;       // njobs + 1
    float ms_last = 0.0f;
};

namespace {

template <typename T>
T* plan_alloc(spg_plan* p, size_t count, const char* what) {
    void* q = nullptr;
    check_cuda(cudaMalloc(&q, std::max<size_t>(count * sizeof(T), 16)), what);
    p->bufs.push_back(q);
    return static_cast<T*>(q);
}

void plan_free(spg_plan* p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    for (void* q : p->bufs) cudaFree(q);
    if (p->hc) cudaFreeHost(p->hc);
    if (p->h_starts) cudaFreeHost(p->h_starts);
    delete p;
}

void plan_build(spg_plan* p, int32_t n, const spg_csr_view* A, const spg_csr_view* B) {
    spg_handle* h = p->h;
    cudaStream_t st = h->stream;
    p->njobs = n;
    p->row_base.assign(n + 1, 0);
    std::vector<Job> jobs(n);
    for (int j = 0; j < n; ++j) {
        check_view(&A[j], "A");
        check_view(&B[j], "B");
        require(A[j].location == SPG_DEVICE && B[j].location == SPG_DEVICE, SPG_INVALID_ARGUMENT,
                "a plan needs device-resident operands");
        require(A[j].cols == B[j].rows, SPG_INVALID_ARGUMENT, "SpGEMM requires A.cols == B.rows");
        p->row_base[j + 1] = p->row_base[j] + A[j].rows;
        p->rows.push_back(A[j].rows);
        p->cols.push_back(B[j].cols);
        auto view = [](const spg_csr_view& m) {
            CsrView v;
            v.rows = m.rows;
            v.cols = m.cols;
            v.nnz = m.nnz;
            v.rp = m.row_ptr;
            v.ci = m.col;
            v.v = m.val;
            return v;
        };
        jobs[j].A = view(A[j]);
        jobs[j].B = view(B[j]);
        jobs[j].row_base = p->row_base[j];
    }
    const int64_t total_rows = p->row_base[n];
    const size_t slots = static_cast<size_t>(total_rows + n);
    int64_t* ub = plan_alloc<int64_t>(p, static_cast<size_t>(total_rows), "plan ub");
    int64_t* cnt = plan_alloc<int64_t>(p, slots, "plan cnt");
    int64_t* nz = plan_alloc<int64_t>(p, slots, "plan nz");
    int64_t* items = plan_alloc<int64_t>(p, static_cast<size_t>(total_rows), "plan items");
    int64_t* d_row_base = plan_alloc<int64_t>(p, static_cast<size_t>(n) + 1, "plan row_base");
    Ctrl* d_ctrl = plan_alloc<Ctrl>(p, 1, "plan ctrl");
    Job* d_jobs = plan_alloc<Job>(p, static_cast<size_t>(n), "plan jobs");
    int64_t* d_jp = plan_alloc<int64_t>(p, static_cast<size_t>(n), "plan job products");
    for (int j = 0; j < n; ++j) {
        jobs[j].ub = ub + p->row_base[j];
        jobs[j].cnt = cnt + p->row_base[j] + j;
        jobs[j].nz = nz + p->row_base[j] + j;
        jobs[j].holes = 1;
    }
    check_cuda(cudaMallocHost(reinterpret_cast<void**>(&p->hc), sizeof(Ctrl)), "plan host ctrl");
    check_cuda(cudaMallocHost(reinterpret_cast<void**>(&p->h_starts), sizeof(int64_t) * (n + 1)), "plan host starts");
    check_cuda(cudaMemsetAsync(cnt, 0, slots * sizeof(int64_t), st), "memset");
    check_cuda(cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), st), "memset");
    check_cuda(cudaMemcpyAsync(d_row_base, p->row_base.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st),
               "H2D");
    check_cuda(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(Job) * n, cudaMemcpyHostToDevice, st), "H2D");
    // structure: row work, bins, the upper-bound offsets
    launch_rowwork(d_jobs, n, d_row_base, total_rows, &d_ctrl->stats, &d_ctrl->err, st);
    launch_bin_offsets(&d_ctrl->stats, d_ctrl->bin_off, st);
    launch_bin_scatter(d_jobs, n, d_row_base, total_rows, d_ctrl->bin_off, d_ctrl->cursor, items, st);
    launch_job_products(d_jobs, n, d_row_base, d_jp, st);
    int64_t* partials = plan_alloc<int64_t>(p, scan_partials_count(static_cast<int64_t>(slots)), "plan partials");
    launch_scan(cnt, static_cast<int64_t>(slots) - 1, partials, st);
    launch_readback(d_ctrl, p->hc, sizeof(Ctrl), st);
    check_cuda(cudaGetLastError(), "plan structure launches");
    p->job_products.assign(n, 0);
    check_cuda(cudaMemcpyAsync(p->job_products.data(), d_jp, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st), "D2H");
    sync(h);
    if (p->hc->err.code) {
        std::string msg;
        const spg_status s = map_err(p->hc->err, msg);
        throw Failure{s, msg};
    }
    const int64_t products = static_cast<int64_t>(p->hc->stats.products);
    const int64_t max_ub = static_cast<int64_t>(p->hc->stats.max_ub);
    require(max_ub < (int64_t{1} << 30), SPG_OVERFLOW, "an output row has more than 2^30 scalar products (engine limit)");
    int64_t bin_count[kNumBins], bin_off[kNumBins + 1];
    for (int b = 0; b < kNumBins; ++b) bin_count[b] = static_cast<int64_t>(p->hc->stats.bin_count[b]);
    for (int b = 0; b <= kNumBins; ++b) bin_off[b] = p->hc->bin_off[b];
    if (h->cfg.hbm_budget_bytes)
        require(static_cast<uint64_t>(products) * 24 <= h->cfg.hbm_budget_bytes, SPG_BUDGET_EXCEEDED,
                "plan footprint exceeds the handle's HBM budget");
    int32_t* tmp_col = plan_alloc<int32_t>(p, static_cast<size_t>(products), "plan C_tmp col");
    double* tmp_val = plan_alloc<double>(p, static_cast<size_t>(products), "plan C_tmp val");
    for (int j = 0; j < n; ++j) {
        jobs[j].c_col = tmp_col;
        jobs[j].c_val = tmp_val;
    }
    check_cuda(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(Job) * n, cudaMemcpyHostToDevice, st), "H2D");
    const SplitTotals split = split_totals(p->hc->stats);
    const size_t scratch_bytes = numeric_scratch_bytes(bin_count, max_ub, split, h->num_sms, true);
    void* scratch = scratch_bytes ? plan_alloc<unsigned char>(p, scratch_bytes, "plan scratch") : nullptr;
    p->col = plan_alloc<int32_t>(p, static_cast<size_t>(products), "plan C col");
    p->val = plan_alloc<double>(p, static_cast<size_t>(products), "plan C val");
    p->rp = plan_alloc<int64_t>(p, slots, "plan C row_ptr");
    std::vector<int64_t> idx(n);
    for (int j = 0; j < n; ++j) idx[j] = p->row_base[j] + j;
    int64_t* d_idx = plan_alloc<int64_t>(p, static_cast<size_t>(n), "plan start index");
    int64_t* d_starts = plan_alloc<int64_t>(p, static_cast<size_t>(n), "plan starts");
    check_cuda(cudaMemcpyAsync(d_idx, idx.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, st), "H2D");
    sync(h);  // idx, jobs copied
    int64_t max_rows = 0;
    for (int32_t r : p->rows) max_rows = std::max<int64_t>(max_rows, r);

    // values: the replayed part
    check_cuda(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed), "begin capture");
    cudaMemsetAsync(nz, 0, slots * sizeof(int64_t), st);
    cudaMemsetAsync(d_ctrl, 0, sizeof(Ctrl), st);
    // the bins on three streams, as in run_products (the fork/join is part of the graph)
    cudaEventRecord(h->fork, st);
    for (cudaStream_t a : h->aux) cudaStreamWaitEvent(a, h->fork, 0);
    for (int b = kNumBins - 1; b >= 1; --b)
        if (bin_count[b])
            launch_numeric(b, d_jobs, items + bin_off[b], bin_count[b], max_ub, split, scratch, scratch_bytes,
                           &d_ctrl->stats, &d_ctrl->err,
                           b <= kLastWarpBin ? st : (b <= kLastSmemBin ? h->aux[0] : h->aux[1]), h->num_sms, true,
                           h->bin_variant[b]);
    for (int i = 0; i < 2; ++i) {
        cudaEventRecord(h->join[i], h->aux[i]);
        cudaStreamWaitEvent(st, h->join[i], 0);
    }
    launch_scan(nz, static_cast<int64_t>(slots) - 1, partials, st);
    launch_compact_holes(d_jobs, n, d_row_base, total_rows, p->col, p->val, st);
    launch_gather(nz, d_idx, d_starts, n, st);
    launch_rebase_jobs(nz, p->rp, d_row_base, n, max_rows, st);
    launch_readback(d_starts, p->h_starts, sizeof(int64_t) * n, st);
    launch_readback(d_ctrl, p->hc, sizeof(Ctrl), st);
    const cudaError_t le = cudaGetLastError();
    const cudaError_t ce = cudaStreamEndCapture(st, &p->graph);
    check_cuda(le, "plan capture launches");
    check_cuda(ce, "end capture");
    check_cuda(cudaGraphInstantiate(&p->exec, p->graph, 0), "graph instantiate");
}

}  // namespace

extern "C" {

spg_status spg_plan_create(spg_handle* h, int32_t n, const spg_csr_view* A, const spg_csr_view* B, spg_plan** plan) {
    return guarded(h, [&] {
        require(plan && n >= 1 && A && B, SPG_INVALID_ARGUMENT, "bad plan arguments");
        *plan = nullptr;
        auto* p = new spg_plan;
        p->h = h;
        try {
            plan_build(p, n, A, B);
        } catch (...) {
            cudaStreamSynchronize(h->stream);
            plan_free(p);
            throw;
        }
        *plan = p;
    });
}

spg_status spg_plan_execute(spg_plan* p, int64_t* nnz) {
    if (!p) return SPG_INVALID_ARGUMENT;
    spg_handle* h = p->h;
    return guarded(h, [&] {
        cudaEventRecord(h->ev[0], h->stream);
        check_cuda(cudaGraphLaunch(p->exec, h->stream), "graph launch");
        cudaEventRecord(h->ev[5], h->stream);
        sync(h);
        if (p->hc->err.code) {
            std::string msg;
            const spg_status s = map_err(p->hc->err, msg);
            throw Failure{s, msg};
        }
        p->nz_total = static_cast<int64_t>(p->hc->stats.nz_total);
        p->starts.assign(p->njobs + 1, 0);
        for (int j = 0; j < p->njobs; ++j) p->starts[j] = p->h_starts[j];
        p->starts[p->njobs] = p->nz_total;
        p->executed = true;
        p->ms_last = elapsed(h->ev[0], h->ev[5]);
        if (nnz)
            for (int j = 0; j < p->njobs; ++j) nnz[j] = p->starts[j + 1] - p->starts[j];
    });
}

spg_status spg_plan_result(const spg_plan* p, int32_t i, spg_csr_result* C) {
    if (!p || !C || i < 0 || i >= p->njobs || !p->executed) return SPG_INVALID_ARGUMENT;
    std::memset(C, 0, sizeof(*C));
    C->rows = p->rows[i];
    C->cols = p->cols[i];
    C->nnz = p->starts[i + 1] - p->starts[i];
    C->row_ptr = p->rp + p->row_base[i] + i;
    C->col = p->col + p->starts[i];
    C->val = p->val + p->starts[i];
    C->location = SPG_DEVICE;
    C->products = p->job_products[i];
    return SPG_OK;
}

float spg_plan_last_ms(const spg_plan* p) { return p ? p->ms_last : 0.0f; }

void spg_plan_destroy(spg_plan* p) {
    if (!p) return;
    cudaSetDevice(p->h->device);
    cudaStreamSynchronize(p->h->stream);
    plan_free(p);
}

void* spg_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void spg_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
