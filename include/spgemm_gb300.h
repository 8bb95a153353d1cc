/* GB300-native SpGEMM engine: C ABI (libspgemm_gb300.so).
 *
 * The engine replaces the local CSR x CSR multiply of malchioman/SpGEMM-hpc-thesis
 * on one GPU.  Matrices use the reference's CsrMatrix layout
 * (src/common/csr_matrix.hpp:43-49): int32 rows/cols, int64 row offsets
 * (rows+1 entries, first 0, last nnz), int32 column indices and FP64 values.
 * Results follow the reference's output contract: every row sorted by column
 * without duplicates, exact +0.0/-0.0 sums dropped, NaN and infinities kept,
 * C.rows = A.rows, C.cols = B.cols.  Every stored value is the sequential FP64
 * sum of its products in the reference's order (A entries, then B entries, in
 * stored order; one rounding per multiply and per add), so results are
 * bit-identical to the reference's serialSpgemm and spgemm().
 *
 * Threading: a handle owns one CUDA stream and its workspace; calls on one
 * handle must not overlap.  Use one handle per host thread.
 *
 * Errors: every call returns an spg_status; spg_last_error(handle) gives the
 * message of the last failure on that handle.  include/spgemm_gb300.hpp maps
 * statuses back to the reference's exception types.
 */
#ifndef SPGEMM_GB300_H
#define SPGEMM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SPG_OK = 0,
    SPG_INVALID_ARGUMENT = 1,      /* shapes, malformed CSR, B column outside B.cols (std::invalid_argument) */
    SPG_OVERFLOW = 2,              /* a count beyond the engine's int64/int32 limits (std::overflow_error) */
    SPG_OUT_OF_RANGE_COLUMN = 3,   /* an A column outside B's rows (std::runtime_error in the reference) */
    SPG_OUT_OF_MEMORY = 4,         /* device allocation failed */
    SPG_BUDGET_EXCEEDED = 5,       /* the request's footprint exceeds the handle's HBM budget */
    SPG_DEVICE_TIMEOUT = 6,        /* reserved: no call of this library returns it -- no kernel waits on
                                      another CTA, a flag or a device; an unfinished request polls
                                      as SPG_NOT_READY */
    SPG_CUDA_ERROR = 7,            /* any other CUDA failure */
    SPG_NOT_READY = 8,             /* spg_poll: the request has not finished */
    SPG_CANCELLED = 9,             /* spg_poll: the request was cancelled */
    SPG_FORMAT_ERROR = 10          /* spg_read_matrix_market: unreadable or malformed file (std::runtime_error) */
} spg_status;

typedef enum { SPG_HOST = 0, SPG_DEVICE = 1 } spg_location;

/* Read-only CSR operand.  `location` says where the three arrays live; host
 * arrays may be pageable or pinned (pinned copies are faster). */
typedef struct {
    int32_t rows, cols;
    int64_t nnz;
    const int64_t* row_ptr;
    const int32_t* col;
    const double* val;
    int32_t location;  /* spg_location */
} spg_csr_view;

/* Result CSR.  The arrays are owned by the library (device memory for
 * SPG_DEVICE results, malloc'd host memory for SPG_HOST results) and are
 * released with spg_result_free. */
typedef struct {
    int32_t rows, cols;
    int64_t nnz;
    int64_t* row_ptr;
    int32_t* col;
    double* val;
    int32_t location;
    int32_t reserved;
    int64_t products;  /* scalar products of this result (FLOP count = 2 * products) */
} spg_csr_result;

/* Output layout of a multiply.  UPPER_BOUND writes every row at the prefix of
 * its scalar-product count and compacts once (12 bytes of scratch per product,
 * one pass over the products); EXACT first counts every row's distinct columns
 * (a second pass over the products, no scratch); AUTO picks UPPER_BOUND unless
 * its scratch would exceed the budget or half of the free device memory. */
typedef enum { SPG_MODE_AUTO = 0, SPG_MODE_EXACT = 1, SPG_MODE_UPPER_BOUND = 2 } spg_mode;

typedef struct {
    int32_t device;             /* CUDA device ordinal */
    int32_t mode;               /* spg_mode */
    uint64_t hbm_budget_bytes;  /* largest device footprint a request may reserve; 0 = no limit */
    int32_t bin_streams;        /* streams the numeric bins of one call spread over: 1, or 3 (0 = 3) */
    int32_t reserved;
} spg_config;

/* Per-phase device times of the last multiply on a handle (CUDA events). */
typedef struct {
    float ms_rowwork, ms_symbolic, ms_scan, ms_numeric, ms_compact, ms_total;
    int64_t products, nnz, rows;
    int64_t bin_rows[20];        /* rows per product-count bin: empty, <=32, 64, 96, 128, 192, 256, 384, 512,
                                    768, 1024, 1536, 2048, 3072, 4096, 6144, 8192, 12288, 16384, heavier */
    int64_t launches;            /* kernels this library launched for the call */
    float ms_numeric_bin[20];    /* per bin (same order as bin_rows): time from the start of the numeric
                                    phase to the end of the bin's launch (bins run on three streams at
                                    once); spg_tune runs them one after the other and times each */
} spg_timings;

typedef struct spg_handle spg_handle;

/* ---- handle ----------------------------------------------------------- */
spg_status spg_config_default(spg_config* config);
spg_status spg_create(const spg_config* config, spg_handle** handle);
void spg_destroy(spg_handle* handle);
const char* spg_last_error(const spg_handle* handle);
const char* spg_status_string(spg_status status);
/* The handle's CUDA stream (a cudaStream_t) for callers that order their own work. */
void* spg_stream(spg_handle* handle);

/* ---- plain product ------------------------------------------------------
 * C = A * B.  Replaces the local multiply
 *   CsrMatrix spgemm(const CsrMatrix& localMatrixA, RowBlock localBBlock,
 *                    const CsrMatrix& localMatrixB, const RemoteSparseRows&, MPI_Comm)
 *   (src/baselines/spgemm_exchange.hpp:37-39; body spgemm_exchange.cpp:258-325)
 * with B entirely local (localBBlock = {0, B.rows}, no halo rows), and its
 * serial twin CsrMatrix serialSpgemm(const CsrMatrix&, const CsrMatrix&)
 *   (src/common/spgemm_common.hpp:80; spgemm_common.cpp:131-178,470-472).
 * Errors: A.cols != B.rows -> SPG_INVALID_ARGUMENT (spgemm_common.cpp:106-110);
 * an A column outside [0, B.rows) -> SPG_OUT_OF_RANGE_COLUMN
 * (spgemm_common.cpp:141-143; the baseline aborts through fail(),
 * spgemm_exchange.cpp:82-85).  `out_location` selects where C is returned. */
spg_status spg_multiply(spg_handle* handle, const spg_csr_view* A, const spg_csr_view* B, int32_t out_location,
                        spg_csr_result* C);

/* C = A * B written into caller host arrays: row_ptr of A.rows+1 entries,
 * col/val of c_capacity entries (nnz(C) <= the scalar-product count, so that
 * count is always enough).  When A has 2^22 entries or more the product runs
 * in row blocks holding 1/32, 1/32, 1/16, then 1/8 of A's entries each; the
 * device->host copy of each finished block runs on a second stream while the
 * later blocks compute, so the transfer of C overlaps the computation.  Page-locked buffers (spg_host_alloc) are needed for the
 * overlap; pageable ones work but copy synchronously.  *c_nnz receives nnz(C);
 * if it exceeds c_capacity the call fails with SPG_BUDGET_EXCEEDED and *c_nnz
 * holds a lower bound of the entries needed.  On any failure (that one, an
 * input error found in a later row block, a CUDA error) the call returns only
 * after the copies of earlier blocks have finished, so the caller may reuse or
 * free its arrays at once.  Results are those of
 * spg_multiply.  Same reference counterpart as spg_multiply: the by-value
 * CsrMatrix return of spgemm() (spgemm_exchange.hpp:37-39). */
spg_status spg_multiply_to_host(spg_handle* handle, const spg_csr_view* A, const spg_csr_view* B, int64_t* c_row_ptr,
                                int32_t* c_col, double* c_val, int64_t c_capacity, int64_t* c_nnz);

/* Copies a device result into caller host buffers of exactly C->rows+1 /
 * C->nnz / C->nnz elements (any of them may be NULL to skip that array). */
spg_status spg_result_download(spg_handle* handle, const spg_csr_result* C, int64_t* row_ptr, int32_t* col,
                               double* val);
spg_status spg_result_free(spg_handle* handle, spg_csr_result* C);

/* Scalar products P = sum over A entries of nnz(B row); the reference's FLOP
 * count is 2P.  Replaces std::int64_t scalarMultiplicationCount(const CsrMatrix&,
 * const CsrMatrix&) (src/common/spgemm_common.hpp:81; spgemm_common.cpp:474-487),
 * with the same errors as spg_multiply. */
spg_status spg_scalar_multiplication_count(spg_handle* handle, const spg_csr_view* A, const spg_csr_view* B,
                                           int64_t* products);

/* Row blocks for multi-GPU row sharding: first_row[0..parts] (parts + 1
 * entries) cut A's rows into `parts` contiguous blocks of about equal scalar
 * products -- first_row[k] is the first row whose preceding products reach
 * floor(k * P / parts), first_row[0] = 0, first_row[parts] = A.rows -- so that
 * G GPUs each multiplying one block against a replicated B get about P / G
 * products each.  Replaces std::vector<RowBlock> partitionRows(int, int)
 * (src/common/spgemm_common.cpp:326-337), which splits by row count; with no
 * products at all the split is by row count as there.  Errors as
 * spg_scalar_multiplication_count. */
spg_status spg_partition_rows(spg_handle* handle, const spg_csr_view* A, const spg_csr_view* B, int32_t parts,
                              int32_t* first_row);

/* Per-phase timings of the last spg_multiply / spg_accum_add on the handle. */
spg_status spg_last_timings(const spg_handle* handle, spg_timings* timings);

/* ---- bin autotuner ----------------------------------------------------------------
 * No reference counterpart.  Several numeric bins have two team shapes (warps
 * per CTA x products per thread); for bins 17 and 18 (8,193-16,384 scalar
 * products per row) the two choices are the threshold above which rows are
 * split into column-range pieces: at 8,192 (default) or at 16,384, the rows in
 * between then running whole, one 16-warp CTA each.  Results are identical,
 * times differ with the workload.  spg_tune multiplies A * B reps times (after one warm-up) with every
 * bin on its default shape, then on its alternative, the bins one after the
 * other; a bin whose alternative's median numeric time was at least 3% lower is
 * a candidate, which is then kept only if, with the bins on their streams as
 * calls run them, the median numeric phase with it is at least 0.5% shorter
 * than without it (2 x (reps + 1) more multiplies per candidate).  The choice
 * stays on the handle for later multiplies, batches, to-host products and plans
 * (spg_get/set_bin_variants save and restore it: 20 entries of 0 or 1). */
typedef struct {
    float ms_bin[2][20];   /* median numeric time per bin: [0] default shapes, [1] alternatives */
    int64_t bin_rows[20];
    int64_t products;
    uint8_t variant[20];   /* the choice now on the handle */
} spg_tune_report;
spg_status spg_tune(spg_handle* handle, const spg_csr_view* A, const spg_csr_view* B, int32_t reps,
                    spg_tune_report* report);
spg_status spg_get_bin_variants(const spg_handle* handle, uint8_t* variants);
spg_status spg_set_bin_variants(spg_handle* handle, const uint8_t* variants);

/* ---- accumulate mode -----------------------------------------------------
 * Replaces trident::LocalAccumulator (src/trident/common/matrix_blocks.hpp:23-32;
 * matrix_blocks.cpp:152-200): begin(rows, cols) <-> the constructor,
 * add(A, B) <-> addProduct (C += A*B, products added after the values already
 * held, each coordinate in order), finish <-> `finish() const` (a copy of the
 * current sum; further add calls may follow), end releases the sum (the
 * destructor).  Shape mismatch (A.rows != rows, B.cols != cols or
 * A.cols != B.rows) -> SPG_INVALID_ARGUMENT (matrix_blocks.cpp:155-157).
 * Exact zeros are absent from the result; dropping them between stages does
 * not change any result, because a later stage's sum starting from +0.0 or
 * from nothing is the same value.  One accumulation per handle at a time. */
spg_status spg_accum_begin(spg_handle* handle, int32_t rows, int32_t cols);
spg_status spg_accum_add(spg_handle* handle, const spg_csr_view* A, const spg_csr_view* B);
spg_status spg_accum_finish(spg_handle* handle, int32_t out_location, spg_csr_result* C);
spg_status spg_accum_end(spg_handle* handle);

/* ---- batched products ------------------------------------------------------
 * n independent products C[i] = A[i] * B[i] in one set of launches per phase
 * (one persistent launch per bin and phase over the concatenated rows of all
 * products).  No reference counterpart: the reference multiplies one product
 * per call (the loop of spgemm() calls in two_sided_spgemm.cpp:146-167).
 * Per-product results and errors are those of spg_multiply; the first failing
 * product's status is returned and no result is produced. */
spg_status spg_multiply_batch(spg_handle* handle, int32_t n, const spg_csr_view* A, const spg_csr_view* B,
                              int32_t out_location, spg_csr_result* C);

/* Scalar products of every product of a batch (one counting pass for all):
 * products[i] = P of A[i] * B[i]; errors as spg_scalar_multiplication_count. */
spg_status spg_scalar_multiplication_count_batch(spg_handle* handle, int32_t n, const spg_csr_view* A,
                                                 const spg_csr_view* B, int64_t* products);

/* ---- Matrix Market input and transposition ----------------------------------------
 * spg_read_matrix_market replaces CsrMatrix readMatrixMarket(const std::string&)
 * (src/common/matrix_market.hpp; matrix_market.cpp:28-145) with the same
 * semantics: coordinate real / integer / pattern matrices, general / symmetric /
 * skew-symmetric / hermitian storage (mirrored entries appended after their
 * entry, negated for skew-symmetric), comments and empty lines skipped, 'D'
 * exponents accepted, entries kept in file order with duplicates, rows built by
 * a stable counting sort.  The entry lines are parsed on all host threads.  The
 * reference's std::runtime_error cases return SPG_FORMAT_ERROR with the message
 * in err (err_len bytes, may be NULL).  The result is in host (malloc) or
 * device memory; release it with spg_result_free on any handle (or
 * spg_csr_release without one). */
spg_status spg_read_matrix_market(const char* path, int32_t out_location, spg_csr_result* C, char* err,
                                  size_t err_len);
/* Frees a result without a handle (host results, or device results when no
 * stream ordering is needed: the device arrays are freed synchronously). */
void spg_csr_release(spg_csr_result* C);
/* C = A^T on the device: C's row j holds A's column j in A's row-major order
 * (the order of a stable sort by column; Gustavson's permuted transposition,
 * the classical companion of the row-wise product the reference cites in
 * docs/sources.md).  No reference counterpart: it forms R^T of the Galerkin
 * chain R A R^T on the device. */
spg_status spg_transpose(spg_handle* handle, const spg_csr_view* A, int32_t out_location, spg_csr_result* C);

/* ---- validation (the reference's Full and Partial modes, on the GPU) -------------
 * Replaces validateProduct(A, B, C, ValidationMode::Full / Partial)
 * (src/common/spgemm_common.cpp:720-851 validateFullStreaming, :541-572
 * buildPartialReference / comparePartialReference) without their caches.  Every
 * coordinate of A * B is recomputed by the reference's own algorithm -- one
 * thread per row walks the row's products in stored order into its own hash
 * table -- as the sequential FP64 sum, a double-double sum of the exact
 * products (the reference uses long double), the double-double magnitude sum
 * and the term count; C is then merged against it.  `passed` (Full): every
 * walked coordinate satisfies the roundoff bound of coordinateBound (:663-675)
 * evaluated with upward rounding (reference precision 2^-100 in place of long
 * double's).  `partial_passed` (Partial): C's row counts equal the counts of
 * nonzero sequential sums.  Malformed or non-finite operands give
 * matrices_ok = 0 and passed = 0, as in the reference.  median_rel_error is the
 * midpoint of a histogram bucket (relative resolution 1/16).  The call returns
 * SPG_OK whenever the check ran, whatever its verdict. */
typedef struct {
    int32_t passed, environment_ok, matrices_ok, partial_passed;
    int64_t rejected, row_nnz_mismatches, support_mismatches, reference_nnz, checked_coordinates;
    double max_abs_error;     /* max |c - sequential FP64 sum| */
    double max_error_ratio;   /* max |c - reference| / bound (capped at 1 where accepted) */
    double max_rel_error, median_rel_error;  /* over stored coordinates, against the reference sum */
} spg_full_report;
spg_status spg_validate_full(spg_handle* handle, const spg_csr_view* A, const spg_csr_view* B, const spg_csr_view* C,
                             spg_full_report* report);

/* ---- plans: one sparsity structure, many value sets ------------------------------
 * No reference counterpart.  For products whose operands keep their structure
 * (row offsets and columns) while their values change -- a Galerkin product
 * re-formed after the fine operator's coefficients change, Trident's
 * repeated stage products -- spg_plan_create runs the structure-dependent
 * phases once (row work, bins, upper-bound offsets, every allocation) for the
 * n device-resident products A[i] * B[i], and captures the value-dependent
 * phases (numeric, scan, compaction, per-product offsets) as one CUDA graph.
 * spg_plan_execute replays the graph on the handle's stream with the values
 * the operand arrays hold at that time, waits for it and writes nnz(C_i) to
 * nnz[i] (nnz may be NULL).  Results equal spg_multiply's bit for bit.  The
 * operand arrays must stay valid and keep their structure for the plan's
 * life.  A plan holds 24 bytes per scalar product plus 40 per row.
 * spg_plan_result gives a device view of product i of the last execution
 * (memory owned by the plan: valid until the next execute or destroy; do not
 * pass it to spg_result_free).  spg_plan_last_ms: device time of the last
 * execution.  A handle's plans and calls share its stream: do not use them
 * from different threads at once. */
typedef struct spg_plan spg_plan;
spg_status spg_plan_create(spg_handle* handle, int32_t n, const spg_csr_view* A, const spg_csr_view* B,
                           spg_plan** plan);
spg_status spg_plan_execute(spg_plan* plan, int64_t* nnz);
spg_status spg_plan_result(const spg_plan* plan, int32_t i, spg_csr_result* C);
float spg_plan_last_ms(const spg_plan* plan);
void spg_plan_destroy(spg_plan* plan);

/* ---- serving loop ---------------------------------------------------------------
 * No reference counterpart (the reference runs one product per call).  A
 * server accepts products as they arrive and runs them in batches on one GPU:
 * `lanes` worker threads, each with its own stream, take the longest prefix
 * of the FIFO queue whose footprint fits the free part of the HBM budget (at
 * most max_batch requests and about max_batch_products scalar products) and
 * multiply it as one spg_multiply_batch; while
 * one batch runs, the next lane admits what arrived meanwhile, so batches
 * overlap on the device.  A request's footprint is its upper-bound device
 * memory: 36 bytes per scalar product + 40 bytes per row of A + its staged
 * host operands + 4 MiB; an uncollected device result stays charged (its own
 * size) until spg_poll returns it.  A request that can never fit fails with
 * SPG_BUDGET_EXCEEDED; an input error fails only the request that has it.
 * Results are bit-identical to spg_multiply of the same operands, alone or in
 * any mix.  Operand arrays must stay valid until the request's spg_poll has
 * returned something other than SPG_NOT_READY. */
typedef struct spg_server spg_server;

typedef struct {
    int32_t device;
    int32_t lanes;              /* batches in flight at once (worker threads/streams); default 2 */
    int32_t max_batch;          /* most requests per batch; 1 runs every request alone; default 256 */
    int32_t out_location;       /* where results are delivered (spg_location); default SPG_DEVICE */
    int32_t mode;               /* spg_mode of the products; default SPG_MODE_AUTO */
    int32_t reserved;
    uint64_t hbm_budget_bytes;  /* admission budget for in-flight work; default 150 GB */
    int64_t max_batch_products; /* a batch stops growing past this many scalar products (a lone larger
                                   request still runs), so that a long queue splits over the lanes
                                   and one lane's host work overlaps another's kernels; default 2^28 */
} spg_server_config;

typedef struct {
    double queue_ms;            /* submit -> admitted to a batch */
    double service_ms;          /* admitted -> result ready */
    double latency_ms;          /* submit -> result ready */
    int64_t products;           /* scalar products of the request */
    int64_t footprint_bytes;    /* admission charge */
    int32_t batch_requests;     /* requests in the batch that served it */
    int32_t lane;               /* worker lane that served it (-1: never ran) */
    uint64_t batch_id;          /* the batch that served it (0: never ran) */
    int64_t batch_launches;     /* kernels that batch launched */
    char message[160];          /* error message of a failed request */
} spg_request_info;

spg_status spg_server_config_default(spg_server_config* config);
spg_status spg_server_create(const spg_server_config* config, spg_server** server);
/* Cancels queued requests, waits for running batches, frees undelivered results. */
void spg_server_destroy(spg_server* server);
/* Queues C = A * B; *ticket identifies it for spg_poll / spg_cancel. */
spg_status spg_submit(spg_server* server, const spg_csr_view* A, const spg_csr_view* B, uint64_t* ticket);
/* Waits up to wait_ms (< 0: without limit) for the request.  SPG_NOT_READY:
 * still queued or running (poll again).  Otherwise the request is retired: its
 * status is returned (SPG_OK with *C filled, the request's error, or
 * SPG_CANCELLED) and `info` (may be NULL) describes it. */
spg_status spg_poll(spg_server* server, uint64_t ticket, int32_t wait_ms, spg_csr_result* C,
                    spg_request_info* info);
/* Cancels a queued request (SPG_OK); SPG_NOT_READY if it is already running. */
spg_status spg_cancel(spg_server* server, uint64_t ticket);
/* Frees a result delivered by spg_poll. */
spg_status spg_server_result_free(spg_server* server, spg_csr_result* C);

/* ---- allocation-free product -------------------------------------------------
 * No counterpart in the reference: its multiply always allocates its result.
 * C = A * B for callers that cannot allocate memory when they multiply --
 * code whose device memory is owned entirely by another allocator (a
 * framework's caching pool or an arena reserved at start-up), real-time loops
 * that forbid allocator calls after initialisation, host threads that must not
 * take the allocator's locks.  A and B must be in device memory; the caller
 * passes device arrays for C (row_ptr of A.rows+1 entries, col/val of
 * c_capacity entries) and the stream to run on (NULL: the default stream); no
 * handle is needed.  All scratch lives in one 32 MiB device array that the
 * library reserves, once per GPU, for the life of the process; a product whose
 * scratch would exceed it (roughly: 32 bytes per row of A plus 12 bytes per
 * distinct output coordinate) is rejected with SPG_BUDGET_EXCEEDED, as is an
 * nnz(C) above c_capacity (*c_nnz then holds the nnz needed).  The first call
 * on a device looks up the array's device address and is a warm-up: under
 * CUDA's lazy module loading the first launch of each kernel loads its code,
 * which may reserve device memory, so a caller that must see no change in
 * device memory makes one call at start-up.  No call, first or later, may be
 * made on a stream that is being captured: every call waits for its stream and
 * reads control values back through pageable host memory (such a stream is
 * rejected with SPG_INVALID_ARGUMENT).  The stream must belong to the current
 * device.  Calls share the array: calls that overlap on the GPU race and must
 * be serialised by the caller.  Results are those of spg_multiply.  The call
 * returns after the stream has finished the product; `err` (err_len bytes, may
 * be NULL) receives a message on failure. */
spg_status spg_multiply_noalloc(const spg_csr_view* A, const spg_csr_view* B, void* stream, int64_t* c_row_ptr,
                                int32_t* c_col, double* c_val, int64_t c_capacity, int64_t* c_nnz, char* err,
                                size_t err_len);

/* ---- host staging helpers ------------------------------------------------- */
/* Page-locked host memory (fast host<->device copies); free with spg_host_free. */
void* spg_host_alloc(size_t bytes);
void spg_host_free(void* ptr);

#ifdef __cplusplus
}
#endif

#endif /* SPGEMM_GB300_H */
