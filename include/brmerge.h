/*
 * brmerge.h -- C ABI of the GB300 BRMerge SpGEMM library (libbrmerge.so).
 *
 * C = A * B for CSR matrices with int32 indices and double (or float) values,
 * computed on one NVIDIA GB300 GPU by hand-written sm_103a kernels.  The
 * result is identical to the reference's BRMerge-Precise: row pointers and
 * column indices bit-exact, and double values bit-exact because the kernels
 * add the partial products of every output entry in the reference's binary
 * merge-tree order (BRMerge-SpGEMM/inc/spgemm.h:639-707).
 *
 * Inputs must be valid CSR as the reference's reader guarantees
 * (BRMerge-SpGEMM/src/CSR.cpp:454-477): rpt[0] == 0, rpt non-decreasing,
 * columns in range and strictly increasing within each row.  The host
 * drop-ins validate their inputs on the GPU by default; the device-pointer
 * calls validate when brm_set_validate(ctx, 1) is set.
 *
 * Every function returns a brm_status (0 on success) instead of the
 * reference's assert/throw.  A context binds to the device that is current
 * when it is created and orders its work on one CUDA stream (brm_set_stream);
 * inside a call it also uses a second stream of its own, forked from and
 * joined back into that stream with events, so every call stays in order on
 * the caller's stream and can be captured in a CUDA graph.  Separate
 * contexts may run concurrently on separate streams.
 */
#ifndef BRMERGE_H
#define BRMERGE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BRM_VERSION_MAJOR 0
#define BRM_VERSION_MINOR 1

typedef enum brm_status {
    BRM_SUCCESS = 0,
    BRM_ERR_INVALID_VALUE = 1, /* bad argument: null pointer, negative size, A.N != B.M, dtype */
    BRM_ERR_INVALID_CSR = 2,   /* an input violates the CSR invariants */
    BRM_ERR_ALLOC = 3,         /* device or host allocation failed */
    BRM_ERR_CUDA = 4,          /* a CUDA runtime call failed */
    BRM_ERR_OVERFLOW = 5,      /* nnz(C) does not fit int32 */
    BRM_ERR_NOT_PLANNED = 6,   /* brm_numeric without a matching brm_symbolic */
    BRM_ERR_INTERNAL = 7,      /* a device-side invariant failed */
    BRM_ERR_TIMEOUT = 8,       /* a bounded device wait expired */
    BRM_ERR_NO_DEVICE = 9,     /* no CUDA device */
    BRM_ERR_CAPACITY = 10,     /* request larger than a fixed capacity */
    BRM_ERR_FORMAT = 11,       /* malformed MatrixMarket file (brm_read_mtx*) */
    BRM_ERR_IO = 12            /* a file cannot be opened or read */
} brm_status;

typedef enum brm_dtype { BRM_F64 = 0, BRM_F32 = 1 } brm_dtype;

/* Phase times in seconds; the fields mirror Precise_Timing
 * (BRMerge-SpGEMM/inc/Timings.h:26-46).  GPU phases are timed with CUDA
 * events on the call's stream: compute_flop = row analysis and binning,
 * prefix_sum_flop = prefix sums of the mid-row products, load_balance = host
 * read of the bin counts and sizing of the segment buffers, symbolic = exact
 * row nnz (heavy rows cut into balanced segments), prefix_sum_nnz = crpt
 * scan, compute = numeric phase.  Device forms: pre_allocate and allocate_C
 * are host wall times of the output allocations.  Host drop-ins:
 * pre_allocate = host-to-device copies of A and B, allocate_C = result
 * blocks, cleanup = the part of the copy of C back to the host that is not
 * overlapped with the numeric phase.  The phases never sum above total. */
typedef struct brm_precise_timing {
    double pre_allocate;
    double compute_flop;
    double prefix_sum_flop;
    double load_balance;
    double symbolic;
    double prefix_sum_nnz;
    double allocate_C;
    double compute;
    double cleanup;
    double total;
} brm_precise_timing;

/* Mirrors Upper_Timing (BRMerge-SpGEMM/inc/Timings.h:4-24): compute_flop =
 * row analysis, prefix_sum_flop = the row-product scans, load_balance =
 * buffer sizing and heavy-row segment planning, compute = merge into the
 * upper-bound buffer, prefix_sum_nnz = crpt scan, copy = compaction into C;
 * host drop-ins add pre_allocate = copies of A and B and cleanup = copy of
 * C back to the host.  thread is 0 (one GPU, no thread team). */
typedef struct brm_upper_timing {
    double thread;
    double pre_allocate;
    double compute_flop;
    double prefix_sum_flop;
    double load_balance;
    double allocate_hook;
    double compute;
    double prefix_sum_nnz;
    double allocate_C;
    double copy;
    double cleanup;
    double total;
} brm_upper_timing;

/* A CSR matrix in device memory (borrowed, read-only).  Mirrors the fields
 * of the reference's CSR class (BRMerge-SpGEMM/inc/CSR.h:7-28); val points
 * to double or float according to the call's dtype. */
typedef struct brm_csr {
    int M;
    int N;
    int nnz;
    const int *rpt;
    const int *col;
    const void *val;
} brm_csr;

typedef struct brm_context_s *brm_context;

/* ---- context ------------------------------------------------------------ */
int brm_create(brm_context *ctx);
int brm_destroy(brm_context ctx);
/* cudaStream_t passed as void*; NULL selects the legacy default stream. */
int brm_set_stream(brm_context ctx, void *stream);
int brm_set_validate(brm_context ctx, int on);

/* Row-class policy of a context.  The reference balances rows over threads
 * by flop (spgemm.h:496-503); here rows are binned and heavy rows cut into
 * segments, and two thresholds of that are runtime knobs: seg_cut, the
 * products between cuts of a heavy row (256 .. 2688; segments hold at most
 * 3072 products), and mid_flop, the largest row weight of the batched
 * mid-row kernels (128 .. 2048; batches hold at most 4096).  Results do not
 * depend on them, only speed does. */
typedef struct brm_tuning {
    int seg_cut;
    int mid_flop;
    /* products the long-column scratch holds (columns of heavy-row segments
     * with more than eight products, reduced by separate kernels); columns
     * beyond it are reduced inside the segment kernel.  0: 16 Mi, the default;
     * otherwise 1 .. 2^31. */
    long long long_scratch;
} brm_tuning;

/* NULL restores the defaults (2304, 2048, 0); out-of-range values are
 * BRM_ERR_INVALID_VALUE. */
int brm_set_tuning(brm_context ctx, const brm_tuning *t);
int brm_get_tuning(brm_context ctx, brm_tuning *t);

/* Times the one-call Precise form on the caller's own input (n == 1:
 * brm_precise_device on A[0], B[0]; n > 1: brm_batch_precise on the n pairs)
 * under each candidate setting (seg_cut in {2304, 1536, 1152, 768} x mid_flop
 * in {2048, 1024, 512}, best of two runs each after one warm-up), keeps the
 * fastest in the context and returns it in *best (may be NULL).  No
 * counterpart in the reference. */
int brm_autotune(brm_context ctx, brm_dtype dtype, int n, const brm_csr *A, const brm_csr *B,
                 brm_tuning *best);
/* SM version of this library's device code as loaded on the current device
 * (cudaFuncAttributes.binaryVersion: 103 for the sm_103a build).
 * Diagnostics; no counterpart in the reference. */
int brm_device_code_version(int *sm);
/* 1 when the library was built with -DBRM_CHECKED: the device code then
 * checks the index of every data-dependent access (writes into C and the
 * scratch arrays, computed shared-memory slots, gathers from B) against its
 * bound, skips a failing access, and the call returns BRM_ERR_INTERNAL; the
 * first failure's source line (in the library's kernel sources), index and
 * bound are reported by brm_last_check_failure (all 0 when none failed).
 * Diagnostics for testing the kernels without a sanitizer; no counterpart
 * in the reference. */
int brm_checked_build(void);
int brm_last_check_failure(brm_context ctx, int *line, long long *index, long long *bound);
/* Device-side error bits of the last call on this context (diagnostics). */
int brm_last_device_error(brm_context ctx);
const char *brm_status_string(int status);

/* ---- symbolic / numeric split (device pointers) -------------------------- */

/* Symbolic phase: products per row, row binning, exact nnz per C row and
 * crpt (caller-allocated, M+1 ints, device).  *cnnz (host) receives nnz(C);
 * the call synchronises the context stream to return it.  The plan is kept
 * in the context for the next brm_numeric on the same A and B.
 * Replaces spgemm.h:476-578 (compute_flop .. allocate C). */
int brm_symbolic(brm_context ctx, const brm_csr *A, const brm_csr *B, int *crpt, int *cnnz);

/* Numeric phase: fills ccol/cval (caller-allocated, cnnz entries, device)
 * in merge-tree order.  Replaces spgemm.h:580-721. */
int brm_numeric(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                const int *crpt, int *ccol, void *cval);

/* ---- one-call forms (device pointers, callee-allocated outputs) ----------- */

/* BRMerge-Precise: symbolic then numeric.  Outputs are allocated from the
 * context's stream-ordered pool; release them with brm_device_free.
 * Mirrors brmerge_precise (spgemm.h:468-471).  timing may be NULL. */
int brm_precise_device(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                       int **crpt, int **ccol, void **cval, int *cnnz,
                       brm_precise_timing *timing);

/* BRMerge-Upper: merge into an upper-bound buffer at the row-product
 * offsets, scan the real row sizes, compact.  Mirrors brmerge_upper
 * (spgemm.h:220-223); output identical to brm_precise_device. */
int brm_upper_device(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                     int **crpt, int **ccol, void **cval, int *cnnz, brm_upper_timing *timing);

int brm_device_free(brm_context ctx, void *p);

/* ---- host drop-ins: the reference's argument order ------------------------ */

/* brmerge_precise with host arrays (spgemm.h:468-471): A is M x K, B is
 * K x N.  *crpt (M+1), *ccol and *cval (cnnz) are allocated by the callee
 * (the reference allocates them with new[], spgemm.h:575-578) from a cache
 * of page-locked host blocks, so the device-to-host copy runs at the link's
 * bandwidth; release each with brm_free (never free()).  timing may be NULL.
 * Uses a process-wide context on the current device. */
int brm_precise(const int *arpt, const int *acol, const double *aval, const int *brpt,
                const int *bcol, const double *bval, int **crpt, int **ccol, double **cval,
                int M, int K, int N, int *cnnz, brm_precise_timing *timing);
int brm_upper(const int *arpt, const int *acol, const double *aval, const int *brpt,
              const int *bcol, const double *bval, int **crpt, int **ccol, double **cval,
              int M, int K, int N, int *cnnz, brm_upper_timing *timing);
int brm_precise_f32(const int *arpt, const int *acol, const float *aval, const int *brpt,
                    const int *bcol, const float *bval, int **crpt, int **ccol, float **cval,
                    int M, int K, int N, int *cnnz, brm_precise_timing *timing);
int brm_upper_f32(const int *arpt, const int *acol, const float *aval, const int *brpt,
                  const int *bcol, const float *bval, int **crpt, int **ccol, float **cval,
                  int M, int K, int N, int *cnnz, brm_upper_timing *timing);
/* Releases an array returned by a host drop-in (its block goes back to the
 * page-locked cache).  NULL is ignored. */
void brm_free(void *p);

/* Returns the cached page-locked blocks that no result holds to the driver.
 * No counterpart in the reference (whose results are plain new[] arrays).
 * The cache keeps at most BRM_HOST_CACHE_MB (environment, default 16384)
 * MiB of unused blocks. */
void brm_host_cache_release(void);

/* Kernels this library has launched in this process so far (all contexts
 * and threads; the two of brm_compute_flop_noalloc are not counted).  No
 * counterpart in the reference (a CPU library); a caller reads it around a
 * region to count the GPU work the region issued. */
long long brm_kernel_launches(void);

/* ---- batches: many independent products in one pipeline ---------------------- */

/* Result of brm_batch_precise: the n products C_i = A_i * B_i concatenated
 * by rows.  C_i has row_off[i+1] - row_off[i] rows; its row pointers are
 * crpt[row_off[i] .. row_off[i+1]] minus nnz_off[i] (crpt holds offsets into
 * the concatenated ccol/cval), and its columns are C_i's own (0 .. N_i-1).
 * crpt, ccol and cval are device memory owned by the batch (brm_batch_free);
 * row_off and nnz_off are host arrays of n + 1 entries. */
typedef struct brm_batch {
    int n;
    long long rows;       /* sum of M_i */
    long long nnz;        /* sum of nnz(C_i) */
    long long *row_off;   /* host, n + 1 */
    long long *nnz_off;   /* host, n + 1 */
    int *crpt;            /* device, rows + 1 */
    int *ccol;            /* device, nnz */
    void *cval;           /* device, nnz (dtype) */
    int *rpt_local;       /* device, rows + n: C_i's own row pointers (from 0)
                             at rpt_local[row_off[i] + i ..  row_off[i+1] + i] */
} brm_batch;

/* C_i = A_i * B_i (BRMerge-Precise) for n independent pairs of device CSR
 * matrices of one value type, in one pipeline: the pairs form one product of
 * stacked operands (A block-diagonal, the B_i stacked row-wise with their own
 * columns), so the kernels see every row of every pair at once.  Each C_i is
 * bit-identical to brm_precise_device(A_i, B_i).  No counterpart in the
 * reference (one pair per call).  The concatenated rows and entries must
 * each fit int32 (else BRM_ERR_CAPACITY); nnz of all C_i together must fit
 * int32 (else BRM_ERR_OVERFLOW). */
int brm_batch_precise(brm_context ctx, brm_dtype dtype, int n, const brm_csr *A, const brm_csr *B,
                      brm_batch *out);
int brm_batch_free(brm_context ctx, brm_batch *batch);

/* A batch whose structure stays fixed while its values change (the reuse
 * pattern of iterative methods), replayed as one CUDA graph.  Create makes
 * the stacked structure, the symbolic plan and every C_i's row pointers and
 * columns once (in a private context that copies ctx's tuning), computes the
 * values once, and captures the value-dependent part (gathering the pairs'
 * current values, the numeric phase) into a graph.  Launch replays it on `stream` (cudaStream_t as void*,
 * NULL = legacy default stream), waits for it and returns the device-side
 * error status; the pairs' value arrays are read at launch, so the caller
 * updates them in place (ordered before the launch) and relaunches.  *out
 * describes C like brm_batch_precise, owned by the graph: release it only
 * with brm_batch_graph_destroy.  No counterpart in the reference. */
typedef struct brm_batch_graph_s *brm_batch_graph;
int brm_batch_graph_create(brm_context ctx, brm_dtype dtype, int n, const brm_csr *A,
                           const brm_csr *B, brm_batch_graph *graph, brm_batch *out);
int brm_batch_graph_launch(brm_batch_graph graph, void *stream);
int brm_batch_graph_destroy(brm_batch_graph graph);

/* A batch pipeline: brm_batch_precise captured once as a CUDA graph with
 * fixed capacities and launched once per NEW batch, whatever its structure
 * (pairs, sizes, sparsity), as long as it fits the capacities.  Every buffer
 * the batch needs is allocated at creation (the stacked operands padded to
 * the capacities, C sized by the products, the planning's segment, split and
 * scratch buffers), so a run allocates nothing and synchronises the host
 * once: it uploads the batch's table, launches the graph and reads nnz(C),
 * the per-pair offsets and the device error status.  The device compares each
 * batch's products, heavy-row segments, split table and spill scratch with
 * the capacities and stops the pipeline (BRM_ERR_CAPACITY) when one does not
 * fit; so does the host for the pair count and the stacked sizes.  Each C_i
 * is bit-identical to brm_precise_device(A_i, B_i).  No counterpart in the
 * reference (one pair per call). */
typedef struct brm_batch_caps {
    int pairs;             /* pairs per batch */
    long long rows;        /* sum of M_i (rows of all C_i) */
    long long nnz_a;       /* sum of nnz(A_i) */
    long long b_rows;      /* sum of K_i (rows of all B_i) */
    long long nnz_b;       /* sum of nnz(B_i) */
    int cols;              /* largest N_i */
    long long products;    /* sum of intermediate products, <= INT_MAX (bounds nnz of all C_i) */
    long long seg_slots;   /* heavy-row segment descriptors */
    long long table;       /* split-table entries of the heavy rows */
    long long spill_bytes; /* scratch of rows merged in global memory */
} brm_batch_caps;

/* Capacities for batches like the sample (n pairs): the sample is planned
 * and multiplied once on ctx, and every count is scaled by headroom (>= 1). */
int brm_batch_caps_for(brm_context ctx, brm_dtype dtype, int n, const brm_csr *A,
                       const brm_csr *B, double headroom, brm_batch_caps *caps);

typedef struct brm_batch_pipe_s *brm_batch_pipe;
/* Allocates the buffers and captures the graph (in a private context that
 * copies ctx's tuning); all pairs of its batches have the value type dtype. */
int brm_batch_pipe_create(brm_context ctx, brm_dtype dtype, const brm_batch_caps *caps,
                          brm_batch_pipe *pipe);
int brm_batch_pipe_caps(brm_batch_pipe pipe, brm_batch_caps *caps);
/* Runs one batch of n pairs on `stream` (cudaStream_t as void*, NULL = the
 * legacy default stream) and waits for it.  *out describes C like
 * brm_batch_precise, but every array (device and host) belongs to the pipe
 * and stays valid until its next run or its destruction: do not pass it to
 * brm_batch_free.  One run at a time per pipe. */
int brm_batch_pipe_run(brm_batch_pipe pipe, int n, const brm_csr *A, const brm_csr *B,
                       void *stream, brm_batch *out);
int brm_batch_pipe_destroy(brm_batch_pipe pipe);

/* ---- serving: a request loop over batches ---------------------------------- */

/* A server takes C = A * B requests (Precise, device CSR) from any thread.
 * A submit only queues the request.  An admission thread takes all newly
 * queued requests at once, counts their products with one kernel on a
 * high-priority stream, and rejects a request whose upper-bound bytes
 * (brm_upper_bound plus the operands' copies) alone exceed mem_cap_bytes
 * (its wait returns BRM_ERR_CAPACITY; BRM_ERR_INVALID_CSR for a column or a
 * B row pointer that is not valid CSR).  Worker threads, each with its own
 * context and stream, take whatever is admitted (one value type per batch,
 * arrival order, bounds within 16x of the oldest one's, so small requests do
 * not wait behind large ones), reserve the summed bounds while they stay
 * under the cap, and run them as one brm_batch_precise; requests that arrive
 * while batches run wait for the next free worker, and the batches of
 * different workers overlap on the device.  Express workers take only
 * requests whose bound is at most express_bytes and run on the device's
 * highest-priority streams; where the driver offers SM partitions (green
 * contexts), the express workers and the admission run on a set of
 * express_sms SMs of their own and the other workers on the rest, so a large
 * batch's kernels never hold the SMs a small request needs.  A request
 * completes when its batch does.
 * Every result is bit-identical to brm_precise_device on its pair.  No
 * counterpart in the reference (one library call per product). */
typedef struct brm_server_s *brm_server;

typedef struct brm_server_config {
    long long mem_cap_bytes;  /* <= 0: 60 GiB */
    int max_batch;            /* requests per batch, <= 0: 4096 */
    int workers;              /* concurrent batches of any size, <= 0: 2 (at most 16) */
    int express_workers;      /* small-request workers, < 0: none (NULL cfg: 1; at most 16) */
    long long express_bytes;  /* largest bound an express worker takes, <= 0: 64 MiB */
    int express_sms;          /* SMs set apart for the express workers, 0: 16, < 0: none */
} brm_server_config;

typedef struct brm_server_result {
    int status;              /* brm_status of the request */
    int M, N, nnz;
    const int *rpt;          /* device, M + 1 row pointers starting at 0 */
    const int *col;          /* device, nnz */
    const void *val;         /* device, nnz (the request's dtype) */
    double queued_s;         /* submit -> start of its batch */
    double latency_s;        /* submit -> result ready */
    int batch_size;          /* requests in the batch that computed it */
} brm_server_result;

/* On the current device; cfg may be NULL. */
int brm_server_create(const brm_server_config *cfg, brm_server *srv);
/* SMs of the express partition and of the other workers' partition (both
 * 0 when the server runs without SM partitions). */
int brm_server_sms(brm_server srv, int *express_sms, int *other_sms);
/* A and B must stay valid until the request is done.  Returns at once;
 * admission (and a BRM_ERR_CAPACITY rejection) follows asynchronously. */
int brm_server_submit(brm_server srv, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                      long long *ticket);
/* Waits up to timeout_s (< 0: forever; BRM_ERR_TIMEOUT when not done) and
 * fills *res; the arrays stay valid until brm_server_release(ticket). */
int brm_server_wait(brm_server srv, long long ticket, double timeout_s, brm_server_result *res);
int brm_server_release(brm_server srv, long long ticket);
/* Finishes the queued requests, then frees everything (unreleased results
 * included). */
int brm_server_destroy(brm_server srv);

/* ---- hash SpGEMM comparator ----------------------------------------------------- */

/* C = A*B by binned hash SpGEMM with sorted rows (Nagasaka et al., the
 * comparator of the BRMerge paper: Existing-SpGEMM/inc/hash_mult.h:1028-1057,
 * HashSpGEMM<sortOutput = true>).  The structure of C (crpt, ccol) is
 * identical to brm_precise_device; the values are summed in an order the
 * hardware picks, so they equal the merge-tree values only to rounding (the
 * reference compares such results with |d| < 1e-9 or |d| < 1e-9 |v|,
 * BRMerge-SpGEMM/src/CSR.cpp:214-253).  Outputs as brm_precise_device
 * (release with brm_device_free). */
int brm_hash_device(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                    int **crpt, int **ccol, void **cval, int *cnnz);

/* ---- MatrixMarket reader ------------------------------------------------------ */

/* Phase times in seconds of a read: read = file to device (overlapped
 * reads and host-to-device copies), parse = tokenising and number
 * conversion on the device (plus the exact host conversion of the rare
 * tokens the device defers), build = symmetric expansion, sort by (row,
 * column) and row pointers, total = the whole call. */
typedef struct brm_mtx_timing {
    double read;
    double parse;
    double build;
    double total;
} brm_mtx_timing;

/* Reads a MatrixMarket coordinate file into CSR with the semantics of the
 * reference's CSR::construct (BRMerge-SpGEMM/src/CSR.cpp:259-479): banner
 * "%%MatrixMarket matrix coordinate <real|integer|pattern|complex>
 * <general|symmetric|skew-symmetric>", '%' comment lines, the size line
 * "M N nnz" (nnz > 0), then nnz entries read as whitespace-separated tokens
 * (line breaks do not matter; surplus tokens are ignored).  Indices become
 * 0-based, symmetric entries are mirrored off the diagonal (negated for
 * skew-symmetric), pattern values are 1, complex values keep their real
 * part, rows are sorted by column; values are converted with correct
 * rounding (f32 output: the double rounded to float).  Errors: BRM_ERR_IO,
 * BRM_ERR_FORMAT (banner, size line, a token that is not a number, fewer
 * entries than declared, an index out of range, a repeated (row, column),
 * a value that overflows a double), BRM_ERR_OVERFLOW (more than INT_MAX
 * entries after mirroring).  Where the reference reads out of bounds or
 * moves an out-of-range column to another row, these return
 * BRM_ERR_FORMAT.  The body is tokenised and converted on the device.
 *
 * Device form: *rpt (M+1), *col and *val (nnz) come from the context's
 * stream-ordered pool; release each with brm_device_free.  timing may be
 * NULL. */
int brm_read_mtx_device(brm_context ctx, brm_dtype dtype, const char *path, int *M, int *N,
                        int *nnz, int **rpt, int **col, void **val, brm_mtx_timing *timing);

/* Host form (what CSR::construct fills): arrays from the page-locked host
 * cache, released with brm_free; uses the process-wide context. */
int brm_read_mtx(const char *path, brm_dtype dtype, int *M, int *N, int *nnz, int **rpt,
                 int **col, void **val, brm_mtx_timing *timing);

/* ---- helpers ---------------------------------------------------------------- */

/* Intermediate products of A*B (compute_flop, spgemm.h:59-66); GFLOP/s in
 * the reference is 2 * products / time. */
int brm_compute_flop(brm_context ctx, const brm_csr *A, const brm_csr *B, long long *products);

/* Admission estimate: products of A*B and the device bytes an Upper call
 * needs at most (upper-bound C_bar plus C sized by the products). */
int brm_upper_bound(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                    long long *products, long long *bytes);

/* Per-row intermediate products of A*B (device A, B) without allocating any
 * memory.  This entry point has no counterpart in the reference.  It is for
 * callers that may not allocate when they need the count, for example an
 * admission controller sizing a request before it reserves anything.
 * row_flop: optional caller buffer of A->M ints (device) for the per-row
 * counts; *products (host) receives the total.  Reduction scratch is a fixed
 * 512 KB array in device memory shared by all calls: A->M may be at most
 * 4,194,304 rows (BRM_ERR_CAPACITY beyond), and calls that overlap on the GPU
 * race on the scratch.  The first call on each device looks up the scratch's
 * device address, so make it before any stream capture; the address is kept
 * for the life of the process, so do not call this after a cudaDeviceReset
 * of that device.  The call synchronises `stream` (cudaStream_t as void*;
 * NULL = legacy default).  Status: BRM_ERR_INVALID_CSR when A.rpt, a column
 * of A or B.rpt is not valid CSR (a column out of range, a decreasing row
 * pointer); BRM_ERR_OVERFLOW when a row's count exceeds INT_MAX, which valid
 * CSR cannot produce (a row's count is at most nnz(B)) and which therefore
 * means an A row with repeated columns; row_flop is then left unwritten for
 * that row and *products is 0. */
int brm_compute_flop_noalloc(const brm_csr *A, const brm_csr *B, int *row_flop,
                             long long *products, void *stream);

/* Checks the CSR invariants of X on the device (columns must be < ncols).
 * *bad_row = -1 if valid, else the first offending row.  Returns
 * BRM_SUCCESS or BRM_ERR_INVALID_CSR. */
int brm_validate(brm_context ctx, const brm_csr *X, int ncols, int *bad_row);

#ifdef __cplusplus
}
#endif

#endif /* BRMERGE_H */
