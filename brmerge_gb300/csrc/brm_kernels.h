// brm_kernels.h -- host-side launchers of the BRMerge kernels (one GPU; a main stream and an
// optional second stream).
#pragma once

#include <mutex>

#include <cuda_runtime.h>

#include "brm_plan.h"
#include "brmerge.h"

namespace brm {

// The stream and SM count of a context (brm_api.cu).
cudaStream_t context_stream(brm_context ctx);
int context_num_sms(brm_context ctx);

// brm_numeric without its closing synchronisation (it only enqueues work on
// the context stream, so it can be captured into a CUDA graph once every
// buffer it needs has been sized by an earlier numeric call on the same
// plan), and the error-word read that brm_numeric ends with.
int numeric_async(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                  const int *crpt, int *ccol, void *cval);
int read_device_error(brm_context ctx);

// The process-wide context of the host drop-ins (created on first use) and
// the mutex that serialises its users.
std::mutex &shared_context_mutex();
int shared_context(brm_context *out);

// Captured batch pipelines (brm_batch.cu): reserve_pipe grows every buffer
// of ctx to the capacities (not capturable: it allocates); precise_pipe then
// enqueues one whole Precise call on ctx's stream with no host
// synchronisation and no allocation (capturable), the counts of each input
// checked against the capacities on the device.  The mid rows are computed
// with the plan.  Errors and nnz(C) stay in the device counters
// (context_counters) for the caller to read after the stream.
int reserve_pipe(brm_context ctx, brm_dtype dtype, const PipeCaps &caps);
int precise_pipe(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B, int *crpt,
                 int *ccol, void *cval, const PipeCaps &caps);
const Counters *context_counters(brm_context ctx);
// The counters the last planning left on the host (after a synchronised call).
Counters last_plan_counters(brm_context ctx);
// Gives the context's internal second stream the CUDA stream priority
// `priority` (the caller sets the main stream with brm_set_stream), and the
// device bytes an Upper call on an M-row A with `products` products needs at
// most (brm_upper_bound's estimate).
int set_context_priority(brm_context ctx, int priority);
// Sizes the context's persistent grids for `sms` SMs (a context whose streams
// run on a partition of the device's SMs).
int set_context_sms(brm_context ctx, int sms);
long long upper_bound_bytes(brm_dtype dtype, int M, long long products);
// Device-side capacity check of a captured pipeline: stage 0 after the row
// analysis and the mid-row prefix sums, stage 1 after the symbolic phase.
void launch_pipe_admit(const PlanDev &P, int M, const PipeCaps &caps, int stage, cudaStream_t s);
int device_status(int err);

// Counts one kernel launch of this library (brm_kernel_launches reports the
// process-wide total); every launch site calls it right after <<<...>>>.
void count_launch();
// Adds n kernel launches (the kernels of a captured graph at each launch),
// and the process-wide count so far.
void count_launches(long long n);
long long launches_so_far();

// Row analysis: products per row, row bins and lists, total products
// (replaces compute_flop and the static load balance, spgemm.h:31-56, :496-503).
void launch_analyze(const CsrDev &A, const CsrDev &B, const PlanDev &P, cudaStream_t s);

// Mid-row batches: scan of the mid products in row order and the first row
// of every batch (Counters::n_batch batches).
void launch_batches(const PlanDev &P, int M, void *tmp, cudaStream_t s);

// Exclusive scans with out[n] = total.  The int32 form ORs kErrOverflow into
// cnt->err and stores the int64 total in cnt->cnnz (spgemm.h:564-578).
void launch_scan_i32(const int *in, int *out, int n, Counters *cnt, void *tmp, cudaStream_t s);
void launch_scan_i64(const int *in, long long *out, int n, void *tmp, cudaStream_t s);
size_t scan_tmp_bytes(int n);

// Symbolic phase: exact nnz per row (spgemm.h:505-562).  `only_heavy`
// restricts the row CTA pass to rows above kCap products (the Upper path uses
// it only to route rows to the spill path).
void launch_symbolic(const CsrDev &A, const CsrDev &B, const PlanDev &P, int num_sms,
                     bool only_heavy, bool skip_mid, cudaStream_t s);

// Reorders the segment list by row part (rows [pb[p], pb[p+1]), nparts <=
// 16): out holds the parts' segments contiguously, ranges[2p..2p+1] the
// slice of part p.  cnt and fill (nparts ints each) must be zero.
void launch_seg_partition(const PlanDev &P, const int *pb, int nparts, int *cnt, int *fill,
                          int *out, int *ranges, int num_sms, cudaStream_t s);

// Upper compaction: C[crpt[i]..] = C_bar[scan_flop[i]..] (spgemm.h:429-444).
void launch_compact(int dtype, const PlanDev &P, const int *bar_col, const void *bar_val,
                    const int *crpt, int *ccol, void *cval, cudaStream_t s);

// Input validation: row pointers monotone and in range, columns in range and
// strictly increasing per row (the invariants CSR.cpp:454-477 enforces on
// read).  Writes the first offending row (or -1) to *bad_row (device int).
void launch_validate(const CsrDev &X, int ncols, int *bad_row, cudaStream_t s);

}  // namespace brm

namespace brm {
// A second stream for work independent of the main stream's: `fork` is
// recorded on the main stream and waited for by `aux`, `join` recorded on
// `aux` and waited for by the main stream.  aux == nullptr: one stream.
struct Fork {
    cudaStream_t aux = nullptr;
    cudaEvent_t fork = nullptr;
    cudaEvent_t join = nullptr;
};

// Numeric launchers per value type.  mid_col/mid_val (Precise only): the
// scratch written by launch_mid_scratch_*, moved to C instead of running the
// mid-row kernel again.  With a fork, the rows that need no split table
// (copy, warp and mid rows) run on its aux stream beside the heavy-row
// segments; the launcher joins the streams before it returns.
void launch_numeric_f64(bool upper, const CsrDev &A, const CsrDev &B, const PlanDev &P,
                        const int *crpt, int *ccol, void *cval, void *spill_scratch,
                        unsigned long long spill_bytes, const int *mid_col, const void *mid_val,
                        int num_sms, cudaStream_t s, const Fork &fk);
void launch_numeric_f32(bool upper, const CsrDev &A, const CsrDev &B, const PlanDev &P,
                        const int *crpt, int *ccol, void *cval, void *spill_scratch,
                        unsigned long long spill_bytes, const int *mid_col, const void *mid_val,
                        int num_sms, cudaStream_t s, const Fork &fk);

// One-call Precise: the mid rows' values and lengths (P.nnz) computed with
// the plan, into a scratch of P.mid_pre[M] entries (row r at P.mid_pre[r]).
// which: 1 = the batched mid rows and the four-warp group rows, 2 = the warp
// and tile rows, 3 = all (the parts can run on different streams).
void launch_mid_scratch_f64(const CsrDev &A, const CsrDev &B, const PlanDev &P, int *mid_col,
                            void *mid_val, int num_sms, cudaStream_t s, int which);
void launch_mid_scratch_f32(const CsrDev &A, const CsrDev &B, const PlanDev &P, int *mid_col,
                            void *mid_val, int num_sms, cudaStream_t s, int which);
}  // namespace brm
