// brm_api.cu -- host orchestration behind the C ABI in include/brmerge.h.
//
// Phase order follows brmerge_precise (BRMerge-SpGEMM/inc/spgemm.h:468-735)
// and brmerge_upper (spgemm.h:220-457); every phase is a kernel launch on
// the context's stream.  The only host synchronisations are the ones the
// interface needs: nnz(C) after the symbolic phase (the caller allocates C),
// and the error word after the numeric phase.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "brm_check.cuh"
#include "brm_hostpool.h"
#include "brm_kernels.h"
#include "brmerge.h"

namespace {
std::atomic<long long> g_launches{0};
}  // namespace

void brm::count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void brm::count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

long long brm::launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

// CUDA events of a timed call, in stream order: kEvIn before the host-to-device
// copies of a host drop-in; kEvStart .. kEvScan around the planning phases;
// kEvNum0/kEvNum1 around the numeric phase; kEvScan2 after Upper's nnz scan;
// kEvCopy0/kEvCopy1 around Upper's compaction; kEvOut after the last copy
// of C back to the host.
enum TimingEvent : int {
    kEvStart = 0,   // start of the plan
    kEvAna = 1,     // after the row analysis (products per row, bins)
    kEvSym = 2,     // after the symbolic phase
    kEvScan = 3,    // after the crpt (Precise) or scan_flop (Upper) scan
    kEvNum0 = 4,
    kEvNum1 = 5,
    kEvScan2 = 6,
    kEvCopy0 = 7,
    kEvCopy1 = 8,
    kEvPre = 9,     // after the prefix sums of the mid-row products
    kEvSized = 10,  // after the host read of the bin counts and buffer sizing
    kEvIn = 11,
    kEvOut = 12,
    kNumEvents = 13
};
constexpr long long kLongElems = 16ll << 20;  // products in the long-column scratch
// candidates of brm_autotune (heavy-row cut target x mid-row weight limit)
constexpr int kTuneSegCut[] = {brm::kSegCut, brm::kSegCut * 2 / 3, brm::kSegCut / 2,
                                brm::kSegCut / 3};
constexpr int kTuneMidFlop[] = {2048, 1024, 512};

}  // namespace

struct brm_context_s {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    bool validate = false;
    // plan workspace
    void *ws = nullptr;
    size_t ws_bytes = 0;
    int ws_M = -1;
    brm::PlanDev plan{};
    void *scan_tmp = nullptr;
    int *d_bad = nullptr;
    brm::Counters *h_cnt = nullptr;  // pinned mirror of the device counters
    int *h_bad = nullptr;            // pinned
    long long *h_mid = nullptr;      // pinned: entries of the mid-row scratch (batched, warp)
    // per-A-entry list metadata (B-row start and length)
    DevBuf ameta;
    // heavy-row segments: descriptors + written list, the split table and the
    // long-column scratch of the column reducer
    DevBuf segbuf, splitbuf, longbuf;
    // one-call Precise: mid rows computed with the plan (columns, values)
    DevBuf midbuf;
    int *mid_col = nullptr;
    void *mid_val = nullptr;
    bool mid_ready = false;
    // spill scratch
    DevBuf spill;
    // Upper upper-bound buffer
    DevBuf bar_col, bar_val;
    // plan identity (symbolic -> numeric)
    bool planned = false;
    const int *a_rpt = nullptr, *a_col = nullptr, *b_rpt = nullptr, *b_col = nullptr;
    int pM = 0, pK = 0, pN = 0;
    unsigned long long spill_bytes = 0;
    int last_err = 0;
    // device copies for the host drop-ins
    DevBuf io_arpt, io_acol, io_aval, io_brpt, io_bcol, io_bval, io_crpt, io_ccol, io_cval;
    // host drop-in, numeric by row parts: part bounds and the segment list
    // ordered by part (device), and a second stream that copies finished
    // parts of C back while the next part computes
    DevBuf partbuf;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t part_ev[brm::kMaxParts] = {};
    // a second compute stream: the mid rows run on it beside the heavy-row
    // planning, and the copy, warp and mid rows beside the segments
    brm::Fork fork;
    cudaEvent_t ev[kNumEvents] = {};
    long long long_scratch = kLongElems;  // products the long-column scratch holds
};

namespace {

int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess)
        return BRM_SUCCESS;
    if (e == cudaErrorMemoryAllocation)
        return BRM_ERR_ALLOC;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return BRM_ERR_NO_DEVICE;
    return BRM_ERR_CUDA;
}

#define BRM_CK(call)                                  \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) {                      \
            (void)cudaGetLastError();                 \
            return cuda_status(e_);                   \
        }                                             \
    } while (0)

#define BRM_TRY(call)              \
    do {                           \
        int s_ = (call);           \
        if (s_ != BRM_SUCCESS)     \
            return s_;             \
    } while (0)

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// Grows a context buffer to at least `bytes` (25 % headroom when it grows
// again), stream-ordered on the context's stream: the old block is released
// after the work queued before it, and neither call waits for the device, so
// a context never stalls behind other contexts' kernels to grow.  Every use
// of a buffer on the context's second stream is joined back into the main
// stream before the next growth.
int grow(brm_context ctx, DevBuf &b, size_t bytes)
{
    if (bytes <= b.cap && b.p)
        return BRM_SUCCESS;
    size_t want = bytes < 256 ? 256 : bytes;
    if (b.p) {
        want = std::max(want, b.cap + b.cap / 4);
        cudaFreeAsync(b.p, ctx->stream);
        b.p = nullptr;
        b.cap = 0;
    }
    BRM_CK(cudaMallocAsync(&b.p, want, ctx->stream));
    b.cap = want;
    return BRM_SUCCESS;
}

void release(DevBuf &b)
{
    if (b.p)
        cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
}

size_t workspace_bytes(int M)
{
    size_t m = (size_t)(M > 0 ? M : 1);
    size_t b = 0;
    b += a256(4 * m);                       // flop
    b += a256(4 * (m + 1));                 // nnz
    b += a256(4 * (size_t)brm::kNumBins * m);  // rows
    b += a256(4 * m);                       // copy_leaf
    b += a256(m);                           // spill flags
    b += a256(4 * m);                       // spill_rows
    b += a256(8 * m);                       // spill_off
    b += a256(8 * (m + 1));                 // scan_flop
    b += a256(4 * m);                       // mid_flop
    b += a256(8 * (m + 1));                 // mid_pre
    b += a256(4 * m);                       // mw_flop
    b += a256(8 * (m + 1));                 // mw_pre
    b += a256(4 * m);                       // longk_rows
    b += a256(4 * (m + 1));                 // batch_start
    b += a256(8 * m);                       // seg_base
    b += a256(4 * m);                       // seg_n
    b += a256(8 * m);                       // crange
    b += a256(sizeof(brm::Counters));
    b += a256(brm::scan_tmp_bytes((int)m + 1));
    b += a256(4);                           // bad row
    return b;
}

size_t vsize(brm_dtype d) { return d == BRM_F64 ? 8 : 4; }

int ensure_workspace(brm_context ctx, int M)
{
    if (ctx->ws && M <= ctx->ws_M)
        return BRM_SUCCESS;
    if (ctx->ws) {  // stream-ordered, with headroom (see grow)
        M = (int)std::min<long long>(INT_MAX - 1,
                                     std::max<long long>(M, ctx->ws_M + (long long)ctx->ws_M / 4));
        cudaFreeAsync(ctx->ws, ctx->stream);
        ctx->ws = nullptr;
    }
    size_t bytes = workspace_bytes(M);
    BRM_CK(cudaMallocAsync(&ctx->ws, bytes, ctx->stream));
    ctx->ws_bytes = bytes;
    ctx->ws_M = M;
    size_t m = (size_t)(M > 0 ? M : 1);
    unsigned char *p = (unsigned char *)ctx->ws;
    size_t off = 0;
    auto take = [&](size_t n) {
        unsigned char *r = p + off;
        off += a256(n);
        return r;
    };
    brm::PlanDev &P = ctx->plan;
    P.flop = (int *)take(4 * m);
    P.nnz = (int *)take(4 * (m + 1));
    P.rows = (int *)take(4 * (size_t)brm::kNumBins * m);
    P.copy_leaf = (int *)take(4 * m);
    P.spill = (unsigned char *)take(m);
    P.spill_rows = (int *)take(4 * m);
    P.spill_off = (unsigned long long *)take(8 * m);
    P.scan_flop = (long long *)take(8 * (m + 1));
    P.mid_flop = (int *)take(4 * m);
    P.mid_pre = (long long *)take(8 * (m + 1));
    P.mw_flop = (int *)take(4 * m);
    P.mw_pre = (long long *)take(8 * (m + 1));
    P.longk_rows = (int *)take(4 * m);
    P.batch_start = (int *)take(4 * (m + 1));
    P.seg_base = (unsigned long long *)take(8 * m);
    P.seg_n = (int *)take(4 * m);
    P.crange = (int2 *)take(8 * m);
    P.cnt = (brm::Counters *)take(sizeof(brm::Counters));
    ctx->scan_tmp = take(brm::scan_tmp_bytes((int)m + 1));
    ctx->d_bad = (int *)take(4);
    return BRM_SUCCESS;
}

int ensure_ameta(brm_context ctx, int nnzA)
{
    const size_t n = (size_t)(nnzA > 0 ? nnzA : 1);
    BRM_TRY(grow(ctx, ctx->ameta, 8 * n));
    ctx->plan.abs = (int *)ctx->ameta.p;
    ctx->plan.alen = (int *)ctx->ameta.p + n;
    return BRM_SUCCESS;
}

brm::CsrDev to_dev(const brm_csr *X)
{
    brm::CsrDev d;
    d.M = X->M;
    d.N = X->N;
    d.nnz = X->nnz;
    d.rpt = X->rpt;
    d.col = X->col;
    d.val = X->val;
    return d;
}

int check_pair(const brm_csr *A, const brm_csr *B)
{
    if (!A || !B)
        return BRM_ERR_INVALID_VALUE;
    if (A->M < 0 || A->N < 0 || B->M < 0 || B->N < 0 || A->nnz < 0 || B->nnz < 0)
        return BRM_ERR_INVALID_VALUE;
    if (A->N != B->M)
        return BRM_ERR_INVALID_VALUE;
    if (!A->rpt || !B->rpt)
        return BRM_ERR_INVALID_VALUE;
    if ((A->nnz > 0 && !A->col) || (B->nnz > 0 && !B->col))
        return BRM_ERR_INVALID_VALUE;
    return BRM_SUCCESS;
}

int device_err_status(int err)
{
    if (err == 0)
        return BRM_SUCCESS;
    if (err & brm::kErrOverflow)
        return BRM_ERR_OVERFLOW;
    if (err & brm::kErrBadInput)
        return BRM_ERR_INVALID_CSR;
    if (err & brm::kErrCapacity)
        return BRM_ERR_CAPACITY;
    return BRM_ERR_INTERNAL;
}

int validate_one(brm_context ctx, const brm_csr *X, int ncols, int *bad_row)
{
    BRM_TRY(ensure_workspace(ctx, ctx->ws_M > 0 ? ctx->ws_M : 1));
    BRM_CK(cudaMemsetAsync(ctx->d_bad, 0x7f, sizeof(int), ctx->stream));
    brm::launch_validate(to_dev(X), ncols, ctx->d_bad, ctx->stream);
    BRM_CK(cudaGetLastError());
    BRM_CK(cudaMemcpyAsync(ctx->h_bad, ctx->d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    BRM_CK(cudaStreamSynchronize(ctx->stream));
    const int b = *ctx->h_bad;  // 0x7f7f7f7f: the memset pattern, no offending row
    *bad_row = (b == 0x7f7f7f7f) ? -1 : b;
    return *bad_row < 0 ? BRM_SUCCESS : BRM_ERR_INVALID_CSR;
}

int validate_pair(brm_context ctx, const brm_csr *A, const brm_csr *B)
{
    int bad = -1;
    BRM_TRY(validate_one(ctx, A, A->N, &bad));
    BRM_TRY(validate_one(ctx, B, B->N, &bad));
    return BRM_SUCCESS;
}

void ev_record(brm_context ctx, bool on, int i)
{
    if (on)
        cudaEventRecord(ctx->ev[i], ctx->stream);
}

double ev_sec(brm_context ctx, int a, int b)
{
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev[a], ctx->ev[b]) != cudaSuccess)
        return 0.0;
    return ms * 1e-3;
}

// Planning phase fields of the timing structs, from the events of a timed
// plan_phase.  Precise: compute_flop = row analysis and binning,
// prefix_sum_flop = prefix sums of the mid-row products and batch starts,
// load_balance = host read of the bin counts and sizing of the segment and
// scratch buffers, symbolic = exact row nnz (heavy-row planning included),
// prefix_sum_nnz = crpt scan.
void plan_times(brm_context ctx, brm_precise_timing *t)
{
    t->compute_flop = ev_sec(ctx, kEvStart, kEvAna);
    t->prefix_sum_flop = ev_sec(ctx, kEvAna, kEvPre);
    t->load_balance = ev_sec(ctx, kEvPre, kEvSized);
    t->symbolic = ev_sec(ctx, kEvSized, kEvSym);
    t->prefix_sum_nnz = ev_sec(ctx, kEvSym, kEvScan);
}

// Upper (spgemm.h:220-457 has no symbolic pass): compute_flop = row
// analysis, prefix_sum_flop = the mid-row prefix sums and the scan_flop scan,
// load_balance = buffer sizing plus the heavy-row planning that cuts long
// rows into balanced segments.
void plan_times_upper(brm_context ctx, brm_upper_timing *t)
{
    t->compute_flop = ev_sec(ctx, kEvStart, kEvAna);
    t->prefix_sum_flop = ev_sec(ctx, kEvAna, kEvPre) + ev_sec(ctx, kEvSym, kEvScan);
    t->load_balance = ev_sec(ctx, kEvPre, kEvSym);
}

// Analysis + symbolic (+ crpt scan for Precise).  Leaves ctx->h_cnt filled.
// Timed: events kEvStart, kEvAna, kEvPre, kEvSized, kEvSym, kEvScan.
// fused_dtype >= 0 (one-call Precise only): the mid rows are computed here,
// values included, into ctx->midbuf, and the numeric phase only moves them.
int plan_phase(brm_context ctx, const brm_csr *A, const brm_csr *B, int *crpt, bool upper,
               bool timed, int fused_dtype = -1)
{
    const bool fused = fused_dtype >= 0 && !upper;
    ctx->mid_ready = false;
    BRM_TRY(ensure_workspace(ctx, A->M));
    BRM_TRY(ensure_ameta(ctx, A->nnz));
    if (ctx->validate)
        BRM_TRY(validate_pair(ctx, A, B));
    brm::CsrDev a = to_dev(A), b = to_dev(B);
    ctx->plan.M = A->M;
    ctx->plan.r_lo = 0;
    ctx->plan.r_hi = A->M;
    ctx->plan.seg_range = nullptr;
    ctx->plan.live = brm::kLiveAll;
    brm::PlanDev P = ctx->plan;
    cudaStream_t s = ctx->stream;
    ev_record(ctx, timed, kEvStart);
    BRM_CK(cudaMemsetAsync(P.cnt, 0, sizeof(brm::Counters), s));
    brm::launch_analyze(a, b, P, s);
    ev_record(ctx, timed, kEvAna);
    brm::launch_batches(P, A->M, ctx->scan_tmp, s);
    ev_record(ctx, timed, kEvPre);
    // the segment descriptors of heavy rows are sized by the analysis
    BRM_CK(cudaGetLastError());
    BRM_CK(cudaMemcpyAsync(ctx->h_cnt, P.cnt, sizeof(brm::Counters), cudaMemcpyDeviceToHost, s));
    if (fused) {
        BRM_CK(cudaMemcpyAsync(ctx->h_mid, P.mid_pre + A->M, sizeof(long long),
                               cudaMemcpyDeviceToHost, s));
        BRM_CK(cudaMemcpyAsync(ctx->h_mid + 1, P.mw_pre + A->M, sizeof(long long),
                               cudaMemcpyDeviceToHost, s));
    }
    BRM_CK(cudaStreamSynchronize(s));
    {
        // row classes with rows (the analysis has binned every row): the
        // kernels of the others are not launched
        const brm::Counters &hc = *ctx->h_cnt;
        unsigned live = 0;
        for (int b = 0; b < brm::kNumBins; b++)
            if (hc.bin_count[b] > 0)
                live |= brm::live_bit(b);
        // batched mid rows are counted in batches, the longest heavy rows apart
        if (hc.n_batch > 0)
            live |= brm::live_bit(brm::kBinBatch);
        if (hc.n_huge > 0)
            live |= brm::live_bit(brm::kBinHeavy);
        if (live & brm::live_bit(brm::kBinHeavy))
            live |= brm::kLiveSegs;  // until the planning says no row was segmented
        P.live = ctx->plan.live = live;
    }
    if (fused) {
        // batched mid rows at mid_pre[row], warp mid rows after them
        const long long tot = ctx->h_mid[0] + ctx->h_mid[1];
        const size_t n = (size_t)(tot > 0 ? tot : 1);
        const size_t b_col = a256(4 * n);
        BRM_TRY(grow(ctx, ctx->midbuf, b_col + vsize((brm_dtype)fused_dtype) * n));
        ctx->mid_col = (int *)ctx->midbuf.p;
        ctx->mid_val = (unsigned char *)ctx->midbuf.p + b_col;
        P.mid_cap = ctx->plan.mid_cap = (long long)n;
    }
    {
        const size_t cap = (size_t)ctx->h_cnt->seg_cap + 1;
        const size_t b_run = a256(cap * sizeof(brm::SegRun));
        BRM_TRY(grow(ctx, ctx->segbuf, b_run + cap * (sizeof(brm::SegDesc) + sizeof(int))));
        P.run = (brm::SegRun *)ctx->segbuf.p;
        P.seg = (brm::SegDesc *)((unsigned char *)ctx->segbuf.p + b_run);
        P.seg_list = (int *)(P.seg + cap);
        ctx->plan.run = P.run;
        ctx->plan.seg = P.seg;
        ctx->plan.seg_list = P.seg_list;
    }
    ev_record(ctx, timed, kEvSized);
    if (fused) {
        // the batched and four-warp group mid rows (values into the scratch)
        // on the second stream, beside the warp-row counts, the heavy-row
        // planning and then the warp and tile mid rows; the planning is
        // enqueued first, so its longest rows start before the mid rows
        // take the SMs
        const brm::Fork &fk = ctx->fork;
        BRM_CK(cudaEventRecord(fk.fork, s));
        brm::launch_symbolic(a, b, P, ctx->num_sms, upper, fused, s);
        BRM_CK(cudaStreamWaitEvent(fk.aux, fk.fork, 0));
        if (fused_dtype == BRM_F64)
            brm::launch_mid_scratch_f64(a, b, P, ctx->mid_col, ctx->mid_val, ctx->num_sms, fk.aux,
                                        brm::kMidGroups);
        else
            brm::launch_mid_scratch_f32(a, b, P, ctx->mid_col, ctx->mid_val, ctx->num_sms, fk.aux,
                                        brm::kMidGroups);
        BRM_CK(cudaEventRecord(fk.join, fk.aux));
    } else {
        brm::launch_symbolic(a, b, P, ctx->num_sms, upper, fused, s);
    }
    if (fused) {
        if (fused_dtype == BRM_F64)
            brm::launch_mid_scratch_f64(a, b, P, ctx->mid_col, ctx->mid_val, ctx->num_sms, s,
                                        brm::kMidWarps);
        else
            brm::launch_mid_scratch_f32(a, b, P, ctx->mid_col, ctx->mid_val, ctx->num_sms, s,
                                        brm::kMidWarps);
        BRM_CK(cudaStreamWaitEvent(s, ctx->fork.join, 0));
    }
    ev_record(ctx, timed, kEvSym);
    if (upper)
        brm::launch_scan_i64(P.flop, P.scan_flop, A->M, ctx->scan_tmp, s);
    else
        brm::launch_scan_i32(P.nnz, crpt, A->M, P.cnt, ctx->scan_tmp, s);
    ev_record(ctx, timed, kEvScan);
    BRM_CK(cudaGetLastError());
    BRM_CK(cudaMemcpyAsync(ctx->h_cnt, P.cnt, sizeof(brm::Counters), cudaMemcpyDeviceToHost, s));
    BRM_CK(cudaStreamSynchronize(s));
    ctx->last_err = ctx->h_cnt->err;
    BRM_TRY(device_err_status(ctx->h_cnt->err));
    if (ctx->h_cnt->n_seg == 0)
        ctx->plan.live &= ~brm::kLiveSegs;
    ctx->planned = true;
    ctx->a_rpt = A->rpt;
    ctx->a_col = A->col;
    ctx->b_rpt = B->rpt;
    ctx->b_col = B->col;
    ctx->pM = A->M;
    ctx->pK = A->N;
    ctx->pN = B->N;
    ctx->spill_bytes = ctx->h_cnt->spill_bytes;
    ctx->mid_ready = fused;
    return BRM_SUCCESS;
}

bool plan_matches(brm_context ctx, const brm_csr *A, const brm_csr *B)
{
    return ctx->planned && ctx->a_rpt == A->rpt && ctx->a_col == A->col && ctx->b_rpt == B->rpt &&
           ctx->b_col == B->col && ctx->pM == A->M && ctx->pK == A->N && ctx->pN == B->N;
}

// use_mid: take the mid rows from the one-call scratch (plan_phase fused).
// A row part of the numeric phase: rows [r_lo, r_hi) and, when seg_list is
// set, the part's slice seg_range of that reordered segment list.
struct RowPart {
    int r_lo = 0;
    int r_hi = -1;  // -1: every row
    const int *seg_range = nullptr;
    const int *seg_list = nullptr;
};

// Bytes of the long-column scratch for `elems` products.
size_t long_bytes(long long elems, brm_dtype dtype)
{
    const long long cols = elems / 8 + 1024;
    return a256(sizeof(brm::LongCol) * (size_t)cols) + a256(2 * (size_t)elems + 2) +
           vsize(dtype) * (size_t)elems + 8;
}

// Sizes of the numeric phase's buffers: from the planning's counters, or
// the capacities of a captured pipeline (whose buffers are grown ahead).
struct NumSizes {
    unsigned long long table_cap = 0;    // split-table entries
    unsigned long long total_flop = 0;   // products (long-column scratch, C_bar of Upper)
    unsigned long long spill_bytes = 0;  // spill scratch
    long long c_cap = 0;                 // entries of C (Precise)
};

NumSizes planned_sizes(brm_context ctx)
{
    NumSizes z;
    z.table_cap = ctx->h_cnt->table_cap;
    z.total_flop = ctx->h_cnt->total_flop;
    z.spill_bytes = ctx->spill_bytes;
    z.c_cap = ctx->h_cnt->cnnz;
    return z;
}

int numeric_launch(brm_context ctx, brm_dtype dtype, bool upper, const brm_csr *A,
                   const brm_csr *B, const int *crpt, int *ccol, void *cval, bool use_mid = false,
                   const RowPart &part = RowPart(), bool clear_err = true,
                   const NumSizes *sizes = nullptr)
{
    const bool mid = use_mid && ctx->mid_ready && !upper;
    const NumSizes sz = sizes ? *sizes : planned_sizes(ctx);
    if (sz.spill_bytes)
        BRM_TRY(grow(ctx, ctx->spill, sz.spill_bytes));
    cudaStream_t s = ctx->stream;
    brm::PlanDev P = ctx->plan;
    P.r_lo = part.r_lo;
    P.r_hi = part.r_hi < 0 ? A->M : part.r_hi;
    P.c_cap = upper ? (long long)sz.total_flop : sz.c_cap;
    P.seg_range = part.seg_range;
    if (part.seg_list)
        P.seg_list = (int *)part.seg_list;
    // work_num and (unless the errors of earlier parts must survive) err
    BRM_CK(cudaMemsetAsync(&P.cnt->work_num, 0, (clear_err ? 2 : 1) * sizeof(int), s));
    BRM_CK(cudaMemsetAsync(&P.cnt->work_bnum, 0, 2 * sizeof(int), s));  // work_bnum, work_seg
    BRM_TRY(grow(ctx, ctx->splitbuf, ((size_t)sz.table_cap + 1) * sizeof(int)));
    P.split = (int *)ctx->splitbuf.p;
    ctx->plan.split = P.split;
    {
        // long-column scratch: at most kLongElems products (columns beyond it
        // are reduced inside the segment kernel)
        const long long elems = std::min<long long>((long long)sz.total_flop, ctx->long_scratch);
        const long long cols = elems / 8 + 1024;
        const size_t b_col = a256(sizeof(brm::LongCol) * (size_t)cols);
        const size_t b_leaf = a256(2 * (size_t)elems + 2);
        BRM_TRY(grow(ctx, ctx->longbuf, long_bytes(elems, dtype)));
        unsigned char *q = (unsigned char *)ctx->longbuf.p;
        P.long_col = (brm::LongCol *)q;
        P.long_leaf = (unsigned short *)(q + b_col);
        P.long_val = q + b_col + b_leaf;
        P.long_cap_cols = cols;
        P.long_cap_elems = elems;
        static_assert(offsetof(brm::Counters, long_elems) ==
                          offsetof(brm::Counters, long_cols) + sizeof(unsigned long long),
                      "the two long-column counters are cleared together");
        BRM_CK(cudaMemsetAsync(&P.cnt->long_cols, 0, 2 * sizeof(unsigned long long), s));
    }
    brm::CsrDev a = to_dev(A), b = to_dev(B);
    const int *mcol = mid ? ctx->mid_col : nullptr;
    const void *mval = mid ? ctx->mid_val : nullptr;
    if (dtype == BRM_F64)
        brm::launch_numeric_f64(upper, a, b, P, crpt, ccol, cval, ctx->spill.p, sz.spill_bytes,
                                mcol, mval, ctx->num_sms, s, ctx->fork);
    else
        brm::launch_numeric_f32(upper, a, b, P, crpt, ccol, cval, ctx->spill.p, sz.spill_bytes,
                                mcol, mval, ctx->num_sms, s, ctx->fork);
    BRM_CK(cudaGetLastError());
    return BRM_SUCCESS;
}

int read_err(brm_context ctx)
{
    BRM_CK(cudaMemcpyAsync(&ctx->h_cnt->err, &ctx->plan.cnt->err, sizeof(int),
                           cudaMemcpyDeviceToHost, ctx->stream));
    BRM_CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_cnt->err & brm::kErrChecked) {  // where the checked build stopped an access
        BRM_CK(cudaMemcpyAsync(&ctx->h_cnt->chk_line, &ctx->plan.cnt->chk_line,
                               offsetof(brm::Counters, chk_bound) + sizeof(long long) -
                                   offsetof(brm::Counters, chk_line),
                               cudaMemcpyDeviceToHost, ctx->stream));
        BRM_CK(cudaStreamSynchronize(ctx->stream));
    }
    ctx->last_err = ctx->h_cnt->err;
    return device_err_status(ctx->h_cnt->err);
}

int check_dtype(brm_dtype d) { return (d == BRM_F64 || d == BRM_F32) ? BRM_SUCCESS : BRM_ERR_INVALID_VALUE; }


// Upper after plan_phase(upper): numeric into C_bar, scan of the real row
// sizes, compaction into the caller's C.  Events 4.. as in upper timing.
int upper_numeric_into_bar(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B)
{
    unsigned long long tf = ctx->h_cnt->total_flop;
    BRM_TRY(grow(ctx, ctx->bar_col, (size_t)tf * 4));
    BRM_TRY(grow(ctx, ctx->bar_val, (size_t)tf * vsize(dtype)));
    return numeric_launch(ctx, dtype, true, A, B, nullptr, (int *)ctx->bar_col.p, ctx->bar_val.p);
}

std::mutex g_mu;
brm_context g_ctx = nullptr;

int default_ctx(brm_context *out)
{
    if (!g_ctx) {
        BRM_TRY(brm_create(&g_ctx));
        g_ctx->validate = true;
    }
    *out = g_ctx;
    return BRM_SUCCESS;
}

double now_sec()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Host drop-in numeric phase (Precise, after a fused plan_phase) with the
// copy of C overlapped: the rows are cut into parts of about equal nnz, the
// segment list is grouped by part, and while part p+1 computes on the
// context stream, the copy stream moves part p of ccol/cval to the host
// blocks.  crpt (device io_crpt) is copied first; it also gives the cuts.
int numeric_by_parts(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B, int M,
                     int cnnz, size_t vb, int *h_rpt, int *h_col, void *h_val, int *dcol,
                     void *dval, bool timed)
{
    cudaStream_t s = ctx->stream, cs = ctx->copy_stream;
    const int *d_rpt = (const int *)ctx->io_crpt.p;
    BRM_CK(cudaMemcpyAsync(h_rpt, d_rpt, 4 * ((size_t)M + 1), cudaMemcpyDeviceToHost, s));
    // parts: one per 32 MB of C, at most kHostParts
    constexpr int kHostParts = 8;
    const long long bytes = (long long)cnnz * (long long)(4 + vb);
    const int nparts = (int)std::min<long long>(kHostParts, std::max<long long>(1, bytes >> 25));
    if (nparts <= 1) {
        BRM_TRY(numeric_launch(ctx, dtype, false, A, B, d_rpt, dcol, dval, true));
        ev_record(ctx, timed, kEvNum1);
        if (cnnz > 0) {
            BRM_CK(cudaMemcpyAsync(h_col, dcol, 4 * (size_t)cnnz, cudaMemcpyDeviceToHost, s));
            BRM_CK(cudaMemcpyAsync((char *)h_val, dval, vb * (size_t)cnnz, cudaMemcpyDeviceToHost, s));
        }
        return BRM_SUCCESS;
    }
    BRM_CK(cudaStreamSynchronize(s));  // h_rpt
    int pb[brm::kMaxParts + 1];
    pb[0] = 0;
    for (int p = 1; p < nparts; p++) {
        const long long target = (long long)cnnz * p / nparts;
        const int r = (int)(std::lower_bound(h_rpt, h_rpt + M + 1, (int)target) - h_rpt);
        pb[p] = std::max(pb[p - 1], std::min(r, M));
    }
    pb[nparts] = M;
    // device: pb, cnt, fill, ranges, reordered segment list
    const int nseg = ctx->h_cnt->n_seg;
    const size_t b_small = a256(sizeof(int) * (size_t)(4 * brm::kMaxParts + 4));
    BRM_TRY(grow(ctx, ctx->partbuf, b_small + sizeof(int) * (size_t)(nseg + 1)));
    int *d_pb = (int *)ctx->partbuf.p;
    int *d_cnt = d_pb + (brm::kMaxParts + 1);
    int *d_fill = d_cnt + brm::kMaxParts;
    int *d_ranges = d_fill + brm::kMaxParts;
    int *d_list = (int *)((char *)ctx->partbuf.p + b_small);
    BRM_CK(cudaMemcpyAsync(d_pb, pb, sizeof(int) * (size_t)(nparts + 1), cudaMemcpyHostToDevice, s));
    BRM_CK(cudaMemsetAsync(d_cnt, 0, sizeof(int) * 2 * brm::kMaxParts, s));  // cnt, fill
    // parts run in order of their heavy-row segments, fewest first: the
    // copy then starts after a light part, and the heavy parts compute while
    // earlier parts are copied
    int order[brm::kMaxParts];
    for (int p = 0; p < nparts; p++)
        order[p] = p;
    if (nseg > 0) {
        brm::launch_seg_partition(ctx->plan, d_pb, nparts, d_cnt, d_fill, d_list, d_ranges,
                                  ctx->num_sms, s);
        int hseg[brm::kMaxParts];
        BRM_CK(cudaMemcpyAsync(hseg, d_cnt, sizeof(int) * (size_t)nparts, cudaMemcpyDeviceToHost,
                               s));
        BRM_CK(cudaStreamSynchronize(s));
        std::stable_sort(order, order + nparts, [&](int x, int y) { return hseg[x] < hseg[y]; });
    }
    for (int q = 0; q < nparts; q++) {
        const int p = order[q];
        RowPart part;
        part.r_lo = pb[p];
        part.r_hi = pb[p + 1];
        if (nseg > 0) {
            part.seg_range = d_ranges + 2 * p;
            part.seg_list = d_list;
        }
        BRM_TRY(numeric_launch(ctx, dtype, false, A, B, d_rpt, dcol, dval, true, part, q == 0));
        const long long e0 = h_rpt[pb[p]], e1 = h_rpt[pb[p + 1]];
        if (e1 > e0) {
            BRM_CK(cudaEventRecord(ctx->part_ev[q], s));
            BRM_CK(cudaStreamWaitEvent(cs, ctx->part_ev[q], 0));
            BRM_CK(cudaMemcpyAsync(h_col + e0, dcol + e0, 4 * (size_t)(e1 - e0),
                                   cudaMemcpyDeviceToHost, cs));
            BRM_CK(cudaMemcpyAsync((char *)h_val + vb * (size_t)e0, (char *)dval + vb * (size_t)e0,
                                   vb * (size_t)(e1 - e0), cudaMemcpyDeviceToHost, cs));
        }
    }
    ev_record(ctx, timed, kEvNum1);
    // the context stream waits for the copies (the caller synchronises it)
    cudaEvent_t done = ctx->part_ev[brm::kMaxParts - 1];
    BRM_CK(cudaEventRecord(done, cs));
    BRM_CK(cudaStreamWaitEvent(s, done, 0));
    return BRM_SUCCESS;
}

// Result arrays of a host drop-in, released unless handed to the caller.
template <typename T>
struct HostResult {
    int *rpt = nullptr;
    int *col = nullptr;
    T *val = nullptr;
    bool keep = false;
    ~HostResult()
    {
        if (!keep) {
            brm_free(rpt);
            brm_free(col);
            brm_free(val);
        }
    }
};

// Host drop-in shared by the four host entry points.
template <typename T>
int host_call(bool upper, const int *arpt, const int *acol, const T *aval, const int *brpt,
              const int *bcol, const T *bval, int **crpt_, int **ccol_, T **cval_, int M, int K,
              int N, int *cnnz_, brm_precise_timing *pt, brm_upper_timing *ut)
{
    if (!crpt_ || !ccol_ || !cval_ || !cnnz_ || M < 0 || K < 0 || N < 0 || !arpt || !brpt)
        return BRM_ERR_INVALID_VALUE;
    const brm_dtype dtype = sizeof(T) == 8 ? BRM_F64 : BRM_F32;
    std::lock_guard<std::mutex> lock(g_mu);
    double t_start = now_sec();
    brm_context ctx;
    BRM_TRY(default_ctx(&ctx));
    cudaStream_t s = ctx->stream;
    const int nnzA = arpt[M], nnzB = brpt[K];
    if (nnzA < 0 || nnzB < 0 || (nnzA > 0 && (!acol || !aval)) || (nnzB > 0 && (!bcol || !bval)))
        return BRM_ERR_INVALID_VALUE;
    const bool same = (arpt == brpt && acol == bcol && aval == bval && M == K);
    const bool timed = pt || ut;
    BRM_TRY(grow(ctx, ctx->io_arpt, 4 * ((size_t)M + 1)));
    BRM_TRY(grow(ctx, ctx->io_acol, 4 * (size_t)nnzA));
    BRM_TRY(grow(ctx, ctx->io_aval, sizeof(T) * (size_t)nnzA));
    if (!same) {
        BRM_TRY(grow(ctx, ctx->io_brpt, 4 * ((size_t)K + 1)));
        BRM_TRY(grow(ctx, ctx->io_bcol, 4 * (size_t)nnzB));
        BRM_TRY(grow(ctx, ctx->io_bval, sizeof(T) * (size_t)nnzB));
    }
    ev_record(ctx, timed, kEvIn);
    BRM_CK(cudaMemcpyAsync(ctx->io_arpt.p, arpt, 4 * ((size_t)M + 1), cudaMemcpyHostToDevice, s));
    BRM_CK(cudaMemcpyAsync(ctx->io_acol.p, acol, 4 * (size_t)nnzA, cudaMemcpyHostToDevice, s));
    BRM_CK(cudaMemcpyAsync(ctx->io_aval.p, aval, sizeof(T) * (size_t)nnzA, cudaMemcpyHostToDevice, s));
    brm_csr A{M, K, nnzA, (const int *)ctx->io_arpt.p, (const int *)ctx->io_acol.p, ctx->io_aval.p};
    brm_csr B = A;
    B.N = N;
    if (!same) {
        BRM_CK(cudaMemcpyAsync(ctx->io_brpt.p, brpt, 4 * ((size_t)K + 1), cudaMemcpyHostToDevice, s));
        BRM_CK(cudaMemcpyAsync(ctx->io_bcol.p, bcol, 4 * (size_t)nnzB, cudaMemcpyHostToDevice, s));
        BRM_CK(cudaMemcpyAsync(ctx->io_bval.p, bval, sizeof(T) * (size_t)nnzB, cudaMemcpyHostToDevice, s));
        B = brm_csr{K, N, nnzB, (const int *)ctx->io_brpt.p, (const int *)ctx->io_bcol.p, ctx->io_bval.p};
    }
    BRM_TRY(grow(ctx, ctx->io_crpt, 4 * ((size_t)M + 1)));
    double t_pre = now_sec();
    int cnnz = 0;
    bool copied = false;  // C already copied back part by part
    double t_sym0 = 0, t_sym1 = 0, t_num0 = 0, t_num1 = 0;
    // result arrays: page-locked blocks from the host cache (released by
    // brm_free).  The kernels write C to device buffers, which are copied
    // back: on this part, stores from the kernels straight into mapped host
    // memory ran the numeric phase at the host link's speed and took longer
    // than the device phase plus one copy.
    HostResult<T> R;
    int *dcol = nullptr;
    void *dval = nullptr;
    auto alloc_results = [&]() -> int {
        R.rpt = (int *)brm::host_alloc(4 * ((size_t)M + 1));
        R.col = (int *)brm::host_alloc(4 * (size_t)(cnnz > 0 ? cnnz : 1));
        R.val = (T *)brm::host_alloc(sizeof(T) * (size_t)(cnnz > 0 ? cnnz : 1));
        if (!R.rpt || !R.col || !R.val)
            return BRM_ERR_ALLOC;
        BRM_TRY(grow(ctx, ctx->io_ccol, 4 * (size_t)cnnz));
        BRM_TRY(grow(ctx, ctx->io_cval, sizeof(T) * (size_t)cnnz));
        dcol = (int *)ctx->io_ccol.p;
        dval = ctx->io_cval.p;
        return BRM_SUCCESS;
    };
    if (!upper) {
        // one call: symbolic with the mid rows computed in passing, numeric
        t_sym0 = now_sec();
        BRM_TRY(check_pair(&A, &B));
        ctx->planned = false;
        BRM_TRY(plan_phase(ctx, &A, &B, (int *)ctx->io_crpt.p, false, timed, dtype));
        cnnz = (int)ctx->h_cnt->cnnz;
        t_sym1 = now_sec();
        BRM_TRY(alloc_results());
        t_num0 = now_sec();
        ev_record(ctx, timed, kEvNum0);
        BRM_TRY(numeric_by_parts(ctx, dtype, &A, &B, M, cnnz, sizeof(T), R.rpt, R.col, R.val, dcol,
                                 dval, timed));
        copied = true;
    } else {
        t_sym0 = now_sec();
        BRM_TRY(plan_phase(ctx, &A, &B, nullptr, true, timed));
        ev_record(ctx, timed, kEvNum0);
        BRM_TRY(upper_numeric_into_bar(ctx, dtype, &A, &B));
        ev_record(ctx, timed, kEvNum1);
        brm::launch_scan_i32(ctx->plan.nnz, (int *)ctx->io_crpt.p, M, ctx->plan.cnt, ctx->scan_tmp, s);
        ev_record(ctx, timed, kEvScan2);
        BRM_CK(cudaGetLastError());
        BRM_CK(cudaMemcpyAsync(ctx->h_cnt, ctx->plan.cnt, sizeof(brm::Counters), cudaMemcpyDeviceToHost, s));
        BRM_CK(cudaStreamSynchronize(s));
        ctx->last_err = ctx->h_cnt->err;
        BRM_TRY(device_err_status(ctx->h_cnt->err));
        cnnz = (int)ctx->h_cnt->cnnz;
        t_sym1 = now_sec();
        BRM_TRY(alloc_results());
        t_num0 = now_sec();
        ev_record(ctx, timed, kEvCopy0);
        brm::launch_compact(dtype == BRM_F64 ? 0 : 1, ctx->plan, (const int *)ctx->bar_col.p,
                            ctx->bar_val.p, (const int *)ctx->io_crpt.p, dcol, dval, s);
        ev_record(ctx, timed, kEvCopy1);
        BRM_CK(cudaGetLastError());
    }
    if (!copied) {
        BRM_CK(cudaMemcpyAsync(R.rpt, ctx->io_crpt.p, 4 * ((size_t)M + 1), cudaMemcpyDeviceToHost, s));
        if (cnnz > 0) {
            BRM_CK(cudaMemcpyAsync(R.col, dcol, 4 * (size_t)cnnz, cudaMemcpyDeviceToHost, s));
            BRM_CK(cudaMemcpyAsync(R.val, dval, sizeof(T) * (size_t)cnnz, cudaMemcpyDeviceToHost, s));
        }
    }
    if (timed)  // every copy of C back to the host has been issued on s or joined into it
        BRM_CK(cudaEventRecord(ctx->ev[kEvOut], s));
    BRM_TRY(read_err(ctx));  // synchronises the stream
    t_num1 = now_sec();
    int *crpt = R.rpt, *ccol = R.col;
    T *cval = R.val;
    R.keep = true;
    double t_end = now_sec();
    *crpt_ = crpt;
    *ccol_ = ccol;
    *cval_ = cval;
    *cnnz_ = cnnz;
    (void)t_pre;
    (void)t_sym0;
    // phases from the call's CUDA events; pre_allocate = the host-to-device
    // copies of A and B (plus the workspace set-up before the plan starts),
    // allocate_C = host wall time between the symbolic and numeric phases
    // (result blocks), cleanup = the copy of C back to the host that is not
    // overlapped with the numeric phase
    if (pt) {
        std::memset(pt, 0, sizeof(*pt));
        pt->pre_allocate = ev_sec(ctx, kEvIn, kEvStart);
        plan_times(ctx, pt);
        pt->allocate_C = t_num0 - t_sym1;
        pt->compute = ev_sec(ctx, kEvNum0, kEvNum1);
        pt->cleanup = ev_sec(ctx, kEvNum1, kEvOut);
        pt->total = t_end - t_start;
    }
    if (ut) {
        std::memset(ut, 0, sizeof(*ut));
        ut->pre_allocate = ev_sec(ctx, kEvIn, kEvStart);
        plan_times_upper(ctx, ut);
        ut->compute = ev_sec(ctx, kEvNum0, kEvNum1);
        ut->prefix_sum_nnz = ev_sec(ctx, kEvNum1, kEvScan2);
        ut->allocate_C = t_num0 - t_sym1;
        ut->copy = ev_sec(ctx, kEvCopy0, kEvCopy1);
        ut->cleanup = ev_sec(ctx, kEvCopy1, kEvOut);
        ut->total = t_end - t_start;
    }
    return BRM_SUCCESS;
}

}  // namespace

cudaStream_t brm::context_stream(brm_context ctx) { return ctx->stream; }

int brm::context_num_sms(brm_context ctx) { return ctx->num_sms; }

int brm::numeric_async(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                       const int *crpt, int *ccol, void *cval)
{
    if (!ctx || !crpt)
        return BRM_ERR_INVALID_VALUE;
    BRM_TRY(check_dtype(dtype));
    BRM_TRY(check_pair(A, B));
    if (!plan_matches(ctx, A, B))
        return BRM_ERR_NOT_PLANNED;
    return numeric_launch(ctx, dtype, false, A, B, crpt, ccol, cval);
}

int brm::read_device_error(brm_context ctx) { return read_err(ctx); }

int brm::device_status(int err) { return device_err_status(err); }

const brm::Counters *brm::context_counters(brm_context ctx) { return ctx->plan.cnt; }

int brm::set_context_sms(brm_context ctx, int sms)
{
    ctx->num_sms = std::max(1, sms);
    return BRM_SUCCESS;
}

int brm::set_context_priority(brm_context ctx, int priority)
{
    cudaStream_t s = nullptr;
    BRM_CK(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, priority));
    if (ctx->fork.aux) {
        cudaStreamSynchronize(ctx->fork.aux);
        cudaStreamDestroy(ctx->fork.aux);
    }
    ctx->fork.aux = s;
    return BRM_SUCCESS;
}

long long brm::upper_bound_bytes(brm_dtype dtype, int M, long long products)
{
    const long long s = (long long)vsize(dtype);
    return 2 * products * (4 + s) + 4LL * ((long long)M + 1) + (long long)workspace_bytes(M);
}

brm::Counters brm::last_plan_counters(brm_context ctx) { return *ctx->h_cnt; }

int brm::reserve_pipe(brm_context ctx, brm_dtype dtype, const brm::PipeCaps &c)
{
    if (c.rows < 1 || c.rows >= INT_MAX || c.nnz_a > INT_MAX || c.products > INT_MAX ||
        c.seg_slots < 0 || c.table < 0 || c.spill_bytes < 0)
        return BRM_ERR_CAPACITY;
    BRM_TRY(ensure_workspace(ctx, (int)c.rows));
    BRM_TRY(ensure_ameta(ctx, (int)c.nnz_a));
    {
        const size_t cap = (size_t)c.seg_slots + 1;
        const size_t b_run = a256(cap * sizeof(brm::SegRun));
        BRM_TRY(grow(ctx, ctx->segbuf, b_run + cap * (sizeof(brm::SegDesc) + sizeof(int))));
        ctx->plan.run = (brm::SegRun *)ctx->segbuf.p;
        ctx->plan.seg = (brm::SegDesc *)((unsigned char *)ctx->segbuf.p + b_run);
        ctx->plan.seg_list = (int *)(ctx->plan.seg + cap);
    }
    {
        const size_t n = (size_t)std::max(c.products, 1LL);
        const size_t b_col = a256(4 * n);
        BRM_TRY(grow(ctx, ctx->midbuf, b_col + vsize(dtype) * n));
        ctx->mid_col = (int *)ctx->midbuf.p;
        ctx->mid_val = (unsigned char *)ctx->midbuf.p + b_col;
        ctx->plan.mid_cap = (long long)n;
    }
    BRM_TRY(grow(ctx, ctx->splitbuf, ((size_t)c.table + 1) * sizeof(int)));
    BRM_TRY(grow(ctx, ctx->longbuf, long_bytes(std::min<long long>(c.products, ctx->long_scratch), dtype)));
    if (c.spill_bytes)
        BRM_TRY(grow(ctx, ctx->spill, (size_t)c.spill_bytes));
    BRM_CK(cudaDeviceSynchronize());  // the buffers exist before any capture
    return BRM_SUCCESS;
}

int brm::precise_pipe(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                      int *crpt, int *ccol, void *cval, const brm::PipeCaps &caps)
{
    BRM_TRY(check_dtype(dtype));
    BRM_TRY(check_pair(A, B));
    if (A->M > caps.rows || A->nnz > caps.nnz_a || B->M > caps.b_rows || B->nnz > caps.nnz_b ||
        B->N > caps.cols)
        return BRM_ERR_CAPACITY;
    brm::CsrDev a = to_dev(A), b = to_dev(B);
    ctx->plan.M = A->M;
    ctx->plan.r_lo = 0;
    ctx->plan.r_hi = A->M;
    ctx->plan.seg_range = nullptr;
    ctx->plan.live = brm::kLiveAll;  // the counts are on the device only
    ctx->planned = false;
    const brm::PlanDev P = ctx->plan;
    cudaStream_t s = ctx->stream;
    BRM_CK(cudaMemsetAsync(P.cnt, 0, sizeof(brm::Counters), s));
    brm::launch_analyze(a, b, P, s);
    brm::launch_batches(P, A->M, ctx->scan_tmp, s);
    brm::launch_pipe_admit(P, A->M, caps, 0, s);
    // as in plan_phase: the heavy-row planning is enqueued before the mid
    // rows of the second stream
    const brm::Fork &fk = ctx->fork;
    BRM_CK(cudaEventRecord(fk.fork, s));
    brm::launch_symbolic(a, b, P, ctx->num_sms, false, true, s);
    BRM_CK(cudaStreamWaitEvent(fk.aux, fk.fork, 0));
    if (dtype == BRM_F64)
        brm::launch_mid_scratch_f64(a, b, P, ctx->mid_col, ctx->mid_val, ctx->num_sms, fk.aux,
                                    brm::kMidGroups);
    else
        brm::launch_mid_scratch_f32(a, b, P, ctx->mid_col, ctx->mid_val, ctx->num_sms, fk.aux,
                                    brm::kMidGroups);
    BRM_CK(cudaEventRecord(fk.join, fk.aux));
    if (dtype == BRM_F64)
        brm::launch_mid_scratch_f64(a, b, P, ctx->mid_col, ctx->mid_val, ctx->num_sms, s,
                                    brm::kMidWarps);
    else
        brm::launch_mid_scratch_f32(a, b, P, ctx->mid_col, ctx->mid_val, ctx->num_sms, s,
                                    brm::kMidWarps);
    BRM_CK(cudaStreamWaitEvent(s, fk.join, 0));
    brm::launch_scan_i32(P.nnz, crpt, A->M, P.cnt, ctx->scan_tmp, s);
    brm::launch_pipe_admit(P, A->M, caps, 1, s);
    BRM_CK(cudaGetLastError());
    ctx->mid_ready = true;
    NumSizes z;
    z.table_cap = (unsigned long long)caps.table;
    z.total_flop = (unsigned long long)caps.products;
    z.spill_bytes = (unsigned long long)caps.spill_bytes;
    z.c_cap = caps.products;
    // the plan's error bits (capacity, bad input) must survive the numeric phase
    return numeric_launch(ctx, dtype, false, A, B, crpt, ccol, cval, true, RowPart(), false, &z);
}

std::mutex &brm::shared_context_mutex() { return g_mu; }

int brm::shared_context(brm_context *out) { return default_ctx(out); }

extern "C" {

const char *brm_status_string(int status)
{
    switch (status) {
    case BRM_SUCCESS: return "success";
    case BRM_ERR_INVALID_VALUE: return "invalid argument";
    case BRM_ERR_INVALID_CSR: return "input violates the CSR invariants";
    case BRM_ERR_ALLOC: return "allocation failed";
    case BRM_ERR_CUDA: return "CUDA runtime error";
    case BRM_ERR_OVERFLOW: return "nnz(C) does not fit int32";
    case BRM_ERR_NOT_PLANNED: return "numeric phase without a matching symbolic phase";
    case BRM_ERR_INTERNAL: return "device-side invariant failed";
    case BRM_ERR_TIMEOUT: return "bounded device wait expired";
    case BRM_ERR_NO_DEVICE: return "no CUDA device";
    case BRM_ERR_CAPACITY: return "request exceeds a fixed capacity";
    case BRM_ERR_FORMAT: return "malformed MatrixMarket file";
    case BRM_ERR_IO: return "file cannot be opened or read";
    default: return "unknown status";
    }
}

int brm_create(brm_context *out)
{
    if (!out)
        return BRM_ERR_INVALID_VALUE;
    *out = nullptr;
    int dev = 0;
    BRM_CK(cudaGetDevice(&dev));
    brm_context ctx = new (std::nothrow) brm_context_s();
    if (!ctx)
        return BRM_ERR_ALLOC;
    ctx->device = dev;
    ctx->plan.seg_cut = brm::kSegCut;
    ctx->plan.mid_limit = brm::kMidFlop;
    ctx->plan.live = brm::kLiveAll;
    cudaError_t e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaMallocHost(&ctx->h_cnt, sizeof(brm::Counters));
    if (e == cudaSuccess)
        e = cudaMallocHost(&ctx->h_bad, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMallocHost(&ctx->h_mid, 2 * sizeof(long long));
    for (int i = 0; i < kNumEvents && e == cudaSuccess; i++)
        e = cudaEventCreate(&ctx->ev[i]);
    for (int i = 0; i < brm::kMaxParts && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&ctx->part_ev[i], cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&ctx->fork.aux, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&ctx->fork.fork, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&ctx->fork.join, cudaEventDisableTiming);
    if (e == cudaSuccess) {
        // keep freed stream-ordered allocations cached in this process so
        // repeated calls do not return memory to the driver between calls
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            unsigned long long keep = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        (void)cudaGetLastError();
    }
    if (e != cudaSuccess) {
        brm_destroy(ctx);
        (void)cudaGetLastError();
        return cuda_status(e);
    }
    *out = ctx;
    return BRM_SUCCESS;
}

int brm_destroy(brm_context ctx)
{
    if (!ctx)
        return BRM_ERR_INVALID_VALUE;
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    else
        cudaDeviceSynchronize();
    if (ctx->ws)
        cudaFree(ctx->ws);
    release(ctx->spill);
    release(ctx->ameta);
    release(ctx->segbuf);
    release(ctx->splitbuf);
    release(ctx->longbuf);
    release(ctx->midbuf);
    release(ctx->bar_col);
    release(ctx->bar_val);
    release(ctx->io_arpt);
    release(ctx->io_acol);
    release(ctx->io_aval);
    release(ctx->io_brpt);
    release(ctx->io_bcol);
    release(ctx->io_bval);
    release(ctx->io_crpt);
    release(ctx->io_ccol);
    release(ctx->io_cval);
    if (ctx->h_cnt)
        cudaFreeHost(ctx->h_cnt);
    if (ctx->h_bad)
        cudaFreeHost(ctx->h_bad);
    if (ctx->h_mid)
        cudaFreeHost(ctx->h_mid);
    for (int i = 0; i < kNumEvents; i++)
        if (ctx->ev[i])
            cudaEventDestroy(ctx->ev[i]);
    for (int i = 0; i < brm::kMaxParts; i++)
        if (ctx->part_ev[i])
            cudaEventDestroy(ctx->part_ev[i]);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->fork.aux) {
        cudaStreamSynchronize(ctx->fork.aux);
        cudaStreamDestroy(ctx->fork.aux);
    }
    if (ctx->fork.fork)
        cudaEventDestroy(ctx->fork.fork);
    if (ctx->fork.join)
        cudaEventDestroy(ctx->fork.join);
    release(ctx->partbuf);
    delete ctx;
    return BRM_SUCCESS;
}

int brm_set_stream(brm_context ctx, void *stream)
{
    if (!ctx)
        return BRM_ERR_INVALID_VALUE;
    ctx->stream = (cudaStream_t)stream;
    return BRM_SUCCESS;
}

int brm_set_validate(brm_context ctx, int on)
{
    if (!ctx)
        return BRM_ERR_INVALID_VALUE;
    ctx->validate = on != 0;
    return BRM_SUCCESS;
}

int brm_set_tuning(brm_context ctx, const brm_tuning *t)
{
    if (!ctx)
        return BRM_ERR_INVALID_VALUE;
    const int cut = t ? t->seg_cut : brm::kSegCut;
    const int mid = t ? t->mid_flop : brm::kMidFlop;
    const long long ls = (t && t->long_scratch) ? t->long_scratch : kLongElems;
    if (cut < brm::kMinSegCut || cut > brm::kSegMaxCut || mid < brm::kMinMidFlop ||
        mid > brm::kMidFlop || ls < 1 || ls > (1ll << 31))
        return BRM_ERR_INVALID_VALUE;
    ctx->plan.seg_cut = cut;
    ctx->plan.mid_limit = mid;
    ctx->long_scratch = ls;
    ctx->planned = false;  // a plan made under other knobs is not reused
    return BRM_SUCCESS;
}

int brm_get_tuning(brm_context ctx, brm_tuning *t)
{
    if (!ctx || !t)
        return BRM_ERR_INVALID_VALUE;
    t->seg_cut = ctx->plan.seg_cut;
    t->mid_flop = ctx->plan.mid_limit;
    t->long_scratch = ctx->long_scratch == kLongElems ? 0 : ctx->long_scratch;
    return BRM_SUCCESS;
}

int brm_autotune(brm_context ctx, brm_dtype dtype, int n, const brm_csr *A, const brm_csr *B,
                 brm_tuning *best)
{
    if (!ctx || n < 1 || !A || !B)
        return BRM_ERR_INVALID_VALUE;
    BRM_TRY(check_dtype(dtype));
    brm_tuning keep;
    BRM_TRY(brm_get_tuning(ctx, &keep));
    // one call of the form the caller will use: a single product or a batch
    auto run_once = [&](double *sec) -> int {
        const double t0 = now_sec();
        if (n == 1) {
            int *crpt = nullptr, *ccol = nullptr;
            void *cval = nullptr;
            int cnnz = 0;
            BRM_TRY(brm_precise_device(ctx, dtype, A, B, &crpt, &ccol, &cval, &cnnz, nullptr));
            *sec = now_sec() - t0;
            brm_device_free(ctx, crpt);
            brm_device_free(ctx, ccol);
            brm_device_free(ctx, cval);
        } else {
            brm_batch b;
            BRM_TRY(brm_batch_precise(ctx, dtype, n, A, B, &b));
            *sec = now_sec() - t0;
            brm_batch_free(ctx, &b);
        }
        return BRM_SUCCESS;
    };
    double warm = 0;
    BRM_TRY(brm_set_tuning(ctx, nullptr));
    BRM_TRY(run_once(&warm));  // allocations and caches out of the timed runs
    brm_tuning pick = {brm::kSegCut, brm::kMidFlop, keep.long_scratch};
    double pick_s = 1e300;
    for (const int cut : kTuneSegCut) {
        for (const int mid : kTuneMidFlop) {
            brm_tuning t = {cut, mid, keep.long_scratch};
            BRM_TRY(brm_set_tuning(ctx, &t));
            double s = 1e300;
            for (int rep = 0; rep < 2; rep++) {  // best of two
                double r = 0;
                const int st = run_once(&r);
                if (st != BRM_SUCCESS) {
                    brm_set_tuning(ctx, &keep);
                    return st;
                }
                s = std::min(s, r);
            }
            if (s < pick_s) {
                pick_s = s;
                pick = t;
            }
        }
    }
    BRM_TRY(brm_set_tuning(ctx, &pick));
    if (best)
        *best = pick;
    return BRM_SUCCESS;
}

int brm_last_device_error(brm_context ctx) { return ctx ? ctx->last_err : -1; }

int brm_checked_build(void) { return brm::kCheckedBuild ? 1 : 0; }

int brm_last_check_failure(brm_context ctx, int *line, long long *index, long long *bound)
{
    if (!ctx || !line || !index || !bound)
        return BRM_ERR_INVALID_VALUE;
    const bool failed = (ctx->last_err & brm::kErrChecked) != 0;
    *line = failed ? ctx->h_cnt->chk_line : 0;
    *index = failed ? ctx->h_cnt->chk_idx : 0;
    *bound = failed ? ctx->h_cnt->chk_bound : 0;
    return BRM_SUCCESS;
}

int brm_symbolic(brm_context ctx, const brm_csr *A, const brm_csr *B, int *crpt, int *cnnz)
{
    if (!ctx || !crpt || !cnnz)
        return BRM_ERR_INVALID_VALUE;
    BRM_TRY(check_pair(A, B));
    ctx->planned = false;
    BRM_TRY(plan_phase(ctx, A, B, crpt, false, false));
    *cnnz = (int)ctx->h_cnt->cnnz;
    return BRM_SUCCESS;
}

int brm_numeric(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                const int *crpt, int *ccol, void *cval)
{
    if (!ctx || !crpt)
        return BRM_ERR_INVALID_VALUE;
    BRM_TRY(check_dtype(dtype));
    BRM_TRY(check_pair(A, B));
    if (!plan_matches(ctx, A, B))
        return BRM_ERR_NOT_PLANNED;
    if (ctx->h_cnt->cnnz > 0 && (!ccol || !cval))
        return BRM_ERR_INVALID_VALUE;
    if ((A->nnz > 0 && !A->val) || (B->nnz > 0 && !B->val))
        return BRM_ERR_INVALID_VALUE;
    BRM_TRY(numeric_launch(ctx, dtype, false, A, B, crpt, ccol, cval));
    return read_err(ctx);
}

int brm_precise_device(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                       int **crpt_, int **ccol_, void **cval_, int *cnnz_,
                       brm_precise_timing *timing)
{
    if (!ctx || !crpt_ || !ccol_ || !cval_ || !cnnz_)
        return BRM_ERR_INVALID_VALUE;
    BRM_TRY(check_dtype(dtype));
    BRM_TRY(check_pair(A, B));
    const bool timed = timing != nullptr;
    double t0 = now_sec();
    int *crpt = nullptr;
    BRM_CK(cudaMallocAsync((void **)&crpt, 4 * ((size_t)A->M + 1), ctx->stream));
    double t1 = now_sec();
    ctx->planned = false;
    int st = plan_phase(ctx, A, B, crpt, false, timed, dtype);
    if (st != BRM_SUCCESS) {
        cudaFreeAsync(crpt, ctx->stream);
        return st;
    }
    int cnnz = (int)ctx->h_cnt->cnnz;
    int *ccol = nullptr;
    void *cval = nullptr;
    double t2 = now_sec();
    cudaError_t e = cudaMallocAsync((void **)&ccol, 4 * (size_t)(cnnz > 0 ? cnnz : 1), ctx->stream);
    if (e == cudaSuccess)
        e = cudaMallocAsync(&cval, vsize(dtype) * (size_t)(cnnz > 0 ? cnnz : 1), ctx->stream);
    if (e != cudaSuccess) {
        cudaFreeAsync(crpt, ctx->stream);
        if (ccol)
            cudaFreeAsync(ccol, ctx->stream);
        (void)cudaGetLastError();
        return cuda_status(e);
    }
    double t3 = now_sec();
    ev_record(ctx, timed, kEvNum0);
    st = numeric_launch(ctx, dtype, false, A, B, crpt, ccol, cval, true);
    ev_record(ctx, timed, kEvNum1);
    if (st == BRM_SUCCESS)
        st = read_err(ctx);
    if (st != BRM_SUCCESS) {
        cudaFreeAsync(crpt, ctx->stream);
        cudaFreeAsync(ccol, ctx->stream);
        cudaFreeAsync(cval, ctx->stream);
        return st;
    }
    double t4 = now_sec();
    *crpt_ = crpt;
    *ccol_ = ccol;
    *cval_ = cval;
    *cnnz_ = cnnz;
    if (timed) {
        std::memset(timing, 0, sizeof(*timing));
        timing->pre_allocate = t1 - t0;
        plan_times(ctx, timing);
        timing->allocate_C = t3 - t2;
        timing->compute = ev_sec(ctx, kEvNum0, kEvNum1);
        timing->total = t4 - t0;
    }
    return BRM_SUCCESS;
}

int brm_upper_device(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                     int **crpt_, int **ccol_, void **cval_, int *cnnz_, brm_upper_timing *timing)
{
    if (!ctx || !crpt_ || !ccol_ || !cval_ || !cnnz_)
        return BRM_ERR_INVALID_VALUE;
    BRM_TRY(check_dtype(dtype));
    BRM_TRY(check_pair(A, B));
    const bool timed = timing != nullptr;
    double t0 = now_sec();
    ctx->planned = false;
    BRM_TRY(plan_phase(ctx, A, B, nullptr, true, timed));
    double t1 = now_sec();
    BRM_TRY(grow(ctx, ctx->bar_col, (size_t)ctx->h_cnt->total_flop * 4));
    BRM_TRY(grow(ctx, ctx->bar_val, (size_t)ctx->h_cnt->total_flop * vsize(dtype)));
    double t2 = now_sec();
    int *crpt = nullptr;
    BRM_CK(cudaMallocAsync((void **)&crpt, 4 * ((size_t)A->M + 1), ctx->stream));
    ev_record(ctx, timed, kEvNum0);
    int st = numeric_launch(ctx, dtype, true, A, B, nullptr, (int *)ctx->bar_col.p, ctx->bar_val.p);
    ev_record(ctx, timed, kEvNum1);
    if (st == BRM_SUCCESS) {
        brm::launch_scan_i32(ctx->plan.nnz, crpt, A->M, ctx->plan.cnt, ctx->scan_tmp, ctx->stream);
        ev_record(ctx, timed, kEvScan2);
        cudaError_t e = cudaMemcpyAsync(ctx->h_cnt, ctx->plan.cnt, sizeof(brm::Counters),
                                        cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        st = cuda_status(e);
        if (st == BRM_SUCCESS) {
            ctx->last_err = ctx->h_cnt->err;
            st = device_err_status(ctx->h_cnt->err);
        }
    }
    if (st != BRM_SUCCESS) {
        cudaFreeAsync(crpt, ctx->stream);
        return st;
    }
    int cnnz = (int)ctx->h_cnt->cnnz;
    double t3 = now_sec();
    int *ccol = nullptr;
    void *cval = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&ccol, 4 * (size_t)(cnnz > 0 ? cnnz : 1), ctx->stream);
    if (e == cudaSuccess)
        e = cudaMallocAsync(&cval, vsize(dtype) * (size_t)(cnnz > 0 ? cnnz : 1), ctx->stream);
    if (e != cudaSuccess) {
        cudaFreeAsync(crpt, ctx->stream);
        if (ccol)
            cudaFreeAsync(ccol, ctx->stream);
        (void)cudaGetLastError();
        return cuda_status(e);
    }
    double t4 = now_sec();
    ev_record(ctx, timed, kEvCopy0);
    brm::launch_compact(dtype == BRM_F64 ? 0 : 1, ctx->plan, (const int *)ctx->bar_col.p,
                        ctx->bar_val.p, crpt, ccol, cval, ctx->stream);
    ev_record(ctx, timed, kEvCopy1);
    st = read_err(ctx);
    if (st != BRM_SUCCESS) {
        cudaFreeAsync(crpt, ctx->stream);
        cudaFreeAsync(ccol, ctx->stream);
        cudaFreeAsync(cval, ctx->stream);
        return st;
    }
    double t5 = now_sec();
    *crpt_ = crpt;
    *ccol_ = ccol;
    *cval_ = cval;
    *cnnz_ = cnnz;
    if (timed) {
        std::memset(timing, 0, sizeof(*timing));
        plan_times_upper(ctx, timing);
        timing->allocate_hook = t2 - t1;
        timing->compute = ev_sec(ctx, kEvNum0, kEvNum1);
        timing->prefix_sum_nnz = ev_sec(ctx, kEvNum1, kEvScan2);
        timing->allocate_C = t4 - t3;
        timing->copy = ev_sec(ctx, kEvCopy0, kEvCopy1);
        timing->total = t5 - t0;
    }
    return BRM_SUCCESS;
}

int brm_device_free(brm_context ctx, void *p)
{
    if (!p)
        return BRM_SUCCESS;
    BRM_CK(cudaFreeAsync(p, ctx ? ctx->stream : nullptr));
    return BRM_SUCCESS;
}

int brm_precise(const int *arpt, const int *acol, const double *aval, const int *brpt,
                const int *bcol, const double *bval, int **crpt, int **ccol, double **cval,
                int M, int K, int N, int *cnnz, brm_precise_timing *timing)
{
    return host_call<double>(false, arpt, acol, aval, brpt, bcol, bval, crpt, ccol, cval, M, K, N,
                             cnnz, timing, nullptr);
}

int brm_upper(const int *arpt, const int *acol, const double *aval, const int *brpt,
              const int *bcol, const double *bval, int **crpt, int **ccol, double **cval, int M,
              int K, int N, int *cnnz, brm_upper_timing *timing)
{
    return host_call<double>(true, arpt, acol, aval, brpt, bcol, bval, crpt, ccol, cval, M, K, N,
                             cnnz, nullptr, timing);
}

int brm_precise_f32(const int *arpt, const int *acol, const float *aval, const int *brpt,
                    const int *bcol, const float *bval, int **crpt, int **ccol, float **cval,
                    int M, int K, int N, int *cnnz, brm_precise_timing *timing)
{
    return host_call<float>(false, arpt, acol, aval, brpt, bcol, bval, crpt, ccol, cval, M, K, N,
                            cnnz, timing, nullptr);
}

int brm_upper_f32(const int *arpt, const int *acol, const float *aval, const int *brpt,
                  const int *bcol, const float *bval, int **crpt, int **ccol, float **cval,
                  int M, int K, int N, int *cnnz, brm_upper_timing *timing)
{
    return host_call<float>(true, arpt, acol, aval, brpt, bcol, bval, crpt, ccol, cval, M, K, N,
                            cnnz, nullptr, timing);
}

void brm_free(void *p)
{
    if (p && !brm::host_release(p))
        std::free(p);
}

void brm_host_cache_release(void) { brm::host_trim(); }

long long brm_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int brm_compute_flop(brm_context ctx, const brm_csr *A, const brm_csr *B, long long *products)
{
    if (!ctx || !products)
        return BRM_ERR_INVALID_VALUE;
    BRM_TRY(check_pair(A, B));
    BRM_TRY(ensure_workspace(ctx, A->M));
    BRM_TRY(ensure_ameta(ctx, A->nnz));
    brm::PlanDev P = ctx->plan;
    P.M = A->M;
    ctx->planned = false;
    BRM_CK(cudaMemsetAsync(P.cnt, 0, sizeof(brm::Counters), ctx->stream));
    brm::launch_analyze(to_dev(A), to_dev(B), P, ctx->stream);
    BRM_CK(cudaGetLastError());
    BRM_CK(cudaMemcpyAsync(ctx->h_cnt, P.cnt, sizeof(brm::Counters), cudaMemcpyDeviceToHost,
                           ctx->stream));
    BRM_CK(cudaStreamSynchronize(ctx->stream));
    ctx->last_err = ctx->h_cnt->err;
    BRM_TRY(device_err_status(ctx->h_cnt->err));
    *products = (long long)ctx->h_cnt->total_flop;
    return BRM_SUCCESS;
}

int brm_upper_bound(brm_context ctx, brm_dtype dtype, const brm_csr *A, const brm_csr *B,
                    long long *products, long long *bytes)
{
    if (!bytes)
        return BRM_ERR_INVALID_VALUE;
    BRM_TRY(check_dtype(dtype));
    long long f = 0;
    BRM_TRY(brm_compute_flop(ctx, A, B, &f));
    if (products)
        *products = f;
    *bytes = brm::upper_bound_bytes(dtype, A->M, f);
    return BRM_SUCCESS;
}

int brm_validate(brm_context ctx, const brm_csr *X, int ncols, int *bad_row)
{
    if (!ctx || !X || !bad_row || X->M < 0 || ncols < 0 || !X->rpt)
        return BRM_ERR_INVALID_VALUE;
    if (X->nnz > 0 && !X->col)
        return BRM_ERR_INVALID_VALUE;
    if (X->M == 0) {
        *bad_row = -1;
        return BRM_SUCCESS;
    }
    return validate_one(ctx, X, ncols, bad_row);
}

}  // extern "C"
