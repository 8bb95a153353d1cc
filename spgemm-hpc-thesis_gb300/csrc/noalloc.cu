// spg_multiply_noalloc: C = A * B without allocating any memory.
//
// Some callers cannot allocate at the moment they multiply: code whose device
// memory is owned entirely by another allocator (a framework's caching pool or
// a fixed arena carved out at start-up), real-time loops that forbid allocator
// calls after initialisation, and host threads that must not take the
// allocator's locks.  For them this entry point runs the exact (symbolic)
// variant of the multiply with every scratch buffer -- the per-row counts and
// offsets, the bin lists, the control block, the heavy-row slabs and the
// unsorted C before compaction -- placed in one file-scope device array of
// kNoallocScratchBytes (32 MiB) that the library owns for the life of the
// process on every GPU that loads it.  Inputs and outputs belong to the caller.
//
// The array's host-side name is not a device address; its device address is
// looked up once per device, with that device current, by the first call made
// on that device (cudaGetSymbolAddress).  That first call is also a warm-up:
// under CUDA's lazy module loading the first launch of each kernel loads its
// code, and the driver may reserve device memory for it, so callers that must
// see no change in device memory make one call at start-up.  Later calls with
// the same kinds of rows launch the same kernels and reserve nothing.  No call
// can be made on a stream that is being captured: every call waits for its
// stream and copies through pageable host memory.  The stream must belong to
// the current device.  Every call on a device shares the array and finds the
// previous call's contents in it: the parts that must start at zero are
// cleared on the caller's stream, and calls that overlap on the GPU (other
// streams, other host threads) race on the array and must be serialised by
// the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/spgemm_gb300.h"
#include "spg_common.cuh"

namespace {

using namespace spg;

constexpr size_t kNoallocScratchBytes = size_t{32} << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

struct NoallocCtrl {
    Stats stats;
    ErrWord err;
    int64_t bin_off[kNumBins + 1];
    unsigned long long cursor[kNumBins];
};

// Device address of the scratch array for the current device, looked up once.
unsigned char* scratch_address(int device, std::string& msg) {
    static std::mutex mu;
    static void* addr[kMaxDevices] = {};
    if (device < 0 || device >= kMaxDevices) {
        msg = "device ordinal beyond the supported range";
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            msg = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
            return nullptr;
        }
        addr[device] = p;
    }
    return static_cast<unsigned char*>(addr[device]);
}

// Bump allocator over the scratch array (offsets rounded to 256 bytes).
struct Carve {
    unsigned char* base;
    size_t used = 0;
    template <typename T>
    T* take(size_t count) {
        const size_t at = (used + 255) & ~size_t{255};
        used = at + count * sizeof(T);
        return reinterpret_cast<T*>(base + at);
    }
    bool fits() const { return used <= kNoallocScratchBytes; }
};

spg_status ret(spg_status s, const std::string& msg, char* err, size_t len) {
    if (err && len) {
        std::strncpy(err, msg.c_str(), len - 1);
        err[len - 1] = '\0';
    }
    return s;
}

spg_status from_cuda(cudaError_t e, const char* what, char* err, size_t len) {
    return ret(SPG_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e), err, len);
}

spg_status from_word(const ErrWord& w, char* err, size_t len) {
    char buf[128];
    std::snprintf(buf, sizeof buf, "input check %d failed (detail %lld)", w.where, static_cast<long long>(w.detail));
    if (w.code == kErrColumnRange) return ret(SPG_OUT_OF_RANGE_COLUMN, "A contains a column index outside B's row range", err, len);
    if (w.code == kErrOverflow) return ret(SPG_OVERFLOW, buf, err, len);
    return ret(SPG_INVALID_ARGUMENT, buf, err, len);
}

}  // namespace

extern "C" spg_status spg_multiply_noalloc(const spg_csr_view* A, const spg_csr_view* B, void* stream_ptr,
                                           int64_t* c_row_ptr, int32_t* c_col, double* c_val, int64_t c_capacity,
                                           int64_t* c_nnz, char* err, size_t err_len) {
    if (!A || !B || !c_row_ptr || !c_nnz || c_capacity < 0 || (c_capacity > 0 && (!c_col || !c_val)))
        return ret(SPG_INVALID_ARGUMENT, "NULL argument or negative capacity", err, err_len);
    if (A->location != SPG_DEVICE || B->location != SPG_DEVICE)
        return ret(SPG_INVALID_ARGUMENT, "operands must be in device memory", err, err_len);
    if (A->rows < 0 || A->cols < 0 || B->rows < 0 || B->cols < 0 || A->nnz < 0 || B->nnz < 0 || !A->row_ptr ||
        !B->row_ptr || (A->nnz && (!A->col || !A->val)) || (B->nnz && (!B->col || !B->val)))
        return ret(SPG_INVALID_ARGUMENT, "malformed operand view", err, err_len);
    if (A->cols != B->rows) return ret(SPG_INVALID_ARGUMENT, "SpGEMM requires A.cols == B.rows", err, err_len);
    cudaStream_t st = static_cast<cudaStream_t>(stream_ptr);
    int device = 0;
    cudaError_t ce = cudaGetDevice(&device);
    if (ce != cudaSuccess) return from_cuda(ce, "cudaGetDevice", err, err_len);
    int stream_device = device;
    if (st && (ce = cudaStreamGetDevice(st, &stream_device)) != cudaSuccess)
        return from_cuda(ce, "cudaStreamGetDevice", err, err_len);
    if (stream_device != device)
        return ret(SPG_INVALID_ARGUMENT, "the stream belongs to another device than the current one", err, err_len);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if ((ce = cudaStreamIsCapturing(st, &capture)) != cudaSuccess)
        return from_cuda(ce, "cudaStreamIsCapturing", err, err_len);
    if (capture != cudaStreamCaptureStatusNone)
        return ret(SPG_INVALID_ARGUMENT, "the stream is being captured; this entry point waits for it", err, err_len);
    int num_sms = 0;
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device);
    std::string msg;
    unsigned char* base = scratch_address(device, msg);
    if (!base) return ret(SPG_CUDA_ERROR, msg, err, err_len);

    const int64_t m = A->rows;
    const size_t slots = static_cast<size_t>(m) + 1;
    Carve cv{base};
    Job* d_job = cv.take<Job>(1);
    NoallocCtrl* d_ctrl = cv.take<NoallocCtrl>(1);
    int64_t* d_row_base = cv.take<int64_t>(2);
    int64_t* ub = cv.take<int64_t>(static_cast<size_t>(m));
    int64_t* cnt = cv.take<int64_t>(slots);
    int64_t* nz = cv.take<int64_t>(slots);
    int64_t* items = cv.take<int64_t>(static_cast<size_t>(m));
    int64_t* partials = cv.take<int64_t>(scan_partials_count(static_cast<int64_t>(slots)));
    if (!cv.fits())
        return ret(SPG_BUDGET_EXCEEDED, "A has too many rows for the 32 MiB allocation-free scratch", err, err_len);

    Job job;
    job.A = CsrView{A->rows, A->cols, A->nnz, A->row_ptr, A->col, A->val};
    job.B = CsrView{B->rows, B->cols, B->nnz, B->row_ptr, B->col, B->val};
    job.ub = ub;
    job.cnt = cnt;
    job.nz = nz;
    const int64_t row_base[2] = {0, m};
    NoallocCtrl hc;
    // Clear what every call must find at zero (the array keeps the last call's contents).
    if ((ce = cudaMemsetAsync(d_ctrl, 0, sizeof(NoallocCtrl), st)) != cudaSuccess ||
        (ce = cudaMemsetAsync(cnt, 0, slots * sizeof(int64_t), st)) != cudaSuccess ||
        (ce = cudaMemsetAsync(nz, 0, slots * sizeof(int64_t), st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_row_base, row_base, sizeof row_base, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(d_job, &job, sizeof job, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return from_cuda(ce, "scratch set-up", err, err_len);
    launch_rowwork(d_job, 1, d_row_base, m, &d_ctrl->stats, &d_ctrl->err, st);
    launch_bin_offsets(&d_ctrl->stats, d_ctrl->bin_off, st);
    launch_bin_scatter(d_job, 1, d_row_base, m, d_ctrl->bin_off, d_ctrl->cursor, items, st);
    if ((ce = cudaGetLastError()) != cudaSuccess) return from_cuda(ce, "row work launch", err, err_len);
    if ((ce = cudaMemcpyAsync(&hc, d_ctrl, sizeof hc, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess)
        return from_cuda(ce, "row work", err, err_len);
    if (hc.err.code) return from_word(hc.err, err, err_len);
    const int64_t max_ub = static_cast<int64_t>(hc.stats.max_ub);
    if (max_ub >= (int64_t{1} << 30))
        return ret(SPG_OVERFLOW, "an output row has more than 2^30 scalar products", err, err_len);
    int64_t bin_count[kNumBins];
    for (int b = 0; b < kNumBins; ++b) bin_count[b] = static_cast<int64_t>(hc.stats.bin_count[b]);
    const size_t slab = std::max(symbolic_scratch_bytes(bin_count, max_ub, num_sms),
                                 numeric_scratch_bytes(bin_count, max_ub, SplitTotals{}, num_sms, false, false));
    unsigned char* d_slab = slab ? cv.take<unsigned char>(slab) : nullptr;
    if (!cv.fits())
        return ret(SPG_BUDGET_EXCEEDED, "heavy rows need more than the 32 MiB allocation-free scratch", err, err_len);

    for (int b = 1; b < kNumBins; ++b)
        launch_symbolic(b, d_job, items + hc.bin_off[b], static_cast<int64_t>(hc.stats.bin_count[b]), max_ub, d_slab,
                        slab, &d_ctrl->stats, &d_ctrl->err, st, num_sms);
    launch_scan(cnt, static_cast<int64_t>(slots) - 1, partials, st);
    if ((ce = cudaGetLastError()) != cudaSuccess) return from_cuda(ce, "symbolic launch", err, err_len);
    int64_t total = 0;
    if ((ce = cudaMemcpyAsync(&total, cnt + m, sizeof total, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(&hc.err, &d_ctrl->err, sizeof hc.err, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess)
        return from_cuda(ce, "symbolic phase", err, err_len);
    if (hc.err.code) return from_word(hc.err, err, err_len);
    job.c_col = cv.take<int32_t>(static_cast<size_t>(total));
    job.c_val = cv.take<double>(static_cast<size_t>(total));
    if (!cv.fits())
        return ret(SPG_BUDGET_EXCEEDED, "the product needs more than the 32 MiB allocation-free scratch", err, err_len);
    if ((ce = cudaMemcpyAsync(d_job, &job, sizeof job, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return from_cuda(ce, "job update", err, err_len);
    for (int b = 1; b < kNumBins; ++b)
        launch_numeric(b, d_job, items + hc.bin_off[b], static_cast<int64_t>(hc.stats.bin_count[b]), max_ub, SplitTotals{}, d_slab,
                       slab, &d_ctrl->stats, &d_ctrl->err, st, num_sms, false);
    if ((ce = cudaGetLastError()) != cudaSuccess) return from_cuda(ce, "numeric launch", err, err_len);
    if ((ce = cudaMemcpyAsync(&hc, d_ctrl, sizeof hc, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess)
        return from_cuda(ce, "numeric phase", err, err_len);
    if (hc.err.code) return from_word(hc.err, err, err_len);
    const int64_t nnz = static_cast<int64_t>(hc.stats.nz_total);
    *c_nnz = nnz;
    if (nnz > c_capacity) return ret(SPG_BUDGET_EXCEEDED, "output capacity is smaller than nnz(C) (see c_nnz)", err, err_len);
    // Rows into the caller's arrays: nz scanned gives the final offsets.
    launch_scan(nz, static_cast<int64_t>(slots) - 1, partials, st);
    launch_compact(d_job, static_cast<int>(m), c_col, c_val, st);
    if ((ce = cudaMemcpyAsync(c_row_ptr, nz, slots * sizeof(int64_t), cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
        (ce = cudaGetLastError()) != cudaSuccess || (ce = cudaStreamSynchronize(st)) != cudaSuccess)
        return from_cuda(ce, "compaction", err, err_len);
    return ret(SPG_OK, "", err, err_len);
}
