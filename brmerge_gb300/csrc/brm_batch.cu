// brm_batch.cu -- many independent products C_i = A_i * B_i in one pipeline.
//
// The reference multiplies one pair per call (BRMerge-SpGEMM/inc/spgemm.h:
// 468-735).  Rows of C depend only on their own A row and the B rows it
// names, so a batch of n pairs is one product of stacked operands: A_bd =
// diag(A_1 .. A_n) (A_i's columns shifted by the B rows before it) and B_bd
// = the B_i stacked row-wise with their own columns (N_bd = max N_i).  Every
// row of C_bd is the merge of exactly the lists of its own pair, in the same
// leaf order, over B_i's own columns, so each C_i is bit-identical to a
// separate call and needs no column shift.  The batch runs as one Precise
// pipeline (about thirty kernel launches for all pairs together).
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "brm_common.cuh"
#include "brm_kernels.h"
#include "brmerge.h"

namespace brm {

// One pair on the device: its input views and its offsets in the stacked
// operands (A rows, A entries, B rows = A columns, B entries).
struct BatchPair {
    const int *arpt, *acol, *brpt, *bcol;
    const void *aval, *bval;
    long long row_a, nnz_a, row_b, nnz_b;
    int M, K, N, nnzA, nnzB;
};

// Index of the pair whose [off[i], off[i+1]) holds x (off non-decreasing,
// off[0] = 0, x < off[n]); empty pairs are skipped.
__device__ __forceinline__ int pair_of(const long long *off, int n, long long x)
{
    int lo = 0, hi = n;  // invariant: off[lo] <= x < off[hi]
    while (hi - lo > 1) {
        const int m = (lo + hi) >> 1;
        if (off[m] <= x)
            lo = m;
        else
            hi = m;
    }
    return lo;
}

// Row pointers of A_bd (which = 0) or B_bd (which = 1): one thread per row
// of the concatenation (plus the closing entry).
__global__ void __launch_bounds__(256) k_batch_rows(const BatchPair *pairs, int n,
                                                    const long long *row_off, long long rows,
                                                    int which, int *rpt)
{
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r <= rows;
         r += (long long)gridDim.x * blockDim.x) {
        if (r == rows) {
            const BatchPair &q = pairs[n - 1];
            rpt[r] = which == 0 ? (int)(q.nnz_a + q.nnzA) : (int)(q.nnz_b + q.nnzB);
            continue;
        }
        const int i = pair_of(row_off, n, r);
        const BatchPair &q = pairs[i];
        if (which == 0)
            rpt[r] = (int)(q.nnz_a + q.arpt[r - q.row_a]);
        else
            rpt[r] = (int)(q.nnz_b + q.brpt[r - q.row_b]);
    }
}

// Columns (COLS) and values of A_bd (which = 0) or B_bd (which = 1): one
// thread per entry of the concatenation.  A replay of a fixed structure
// gathers the values alone.
template <typename T, bool COLS>
__global__ void __launch_bounds__(256) k_batch_entries(const BatchPair *pairs, int n,
                                                       const long long *nnz_off, long long nnz,
                                                       int which, int *col, T *val)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nnz;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = pair_of(nnz_off, n, e);
        const BatchPair &q = pairs[i];
        if (which == 0) {
            const long long j = e - q.nnz_a;
            if (COLS)
                col[e] = (int)(q.acol[j] + q.row_b);
            val[e] = ((const T *)q.aval)[j];
        } else {
            const long long j = e - q.nnz_b;
            if (COLS)
                col[e] = q.bcol[j];
            val[e] = ((const T *)q.bval)[j];
        }
    }
}

// Each pair's first entry in C_bd (every pair, including empty ones).
__global__ void __launch_bounds__(256) k_batch_first(const BatchPair *pairs, int n, int rows,
                                                     const int *crpt, long long *nnz_first)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
         i += (long long)gridDim.x * blockDim.x)
        nnz_first[i] = crpt[i < n ? pairs[i].row_a : rows];
}

// Each pair's own row pointers (starting at 0), pair i at out[row_off[i] +
// i .. row_off[i+1] + i].
__global__ void __launch_bounds__(256) k_batch_local_rpt(int n, const long long *row_off,
                                                         long long rows, const int *crpt,
                                                         const long long *first, int *out)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long r = t; r < rows; r += stride) {
        const int i = pair_of(row_off, n, r);
        out[r + i] = (int)(crpt[r] - first[i]);
    }
    for (long long i = t; i < n; i += stride)
        out[row_off[i + 1] + i] = (int)(first[i + 1] - first[i]);
}

}  // namespace brm

namespace {

struct Buf {
    void *p = nullptr;
    size_t cap = 0;
};

int grow_buf(Buf &b, size_t bytes, cudaStream_t s)
{
    if (bytes <= b.cap && b.p)
        return BRM_SUCCESS;
    if (b.p)
        cudaFreeAsync(b.p, s);
    b.p = nullptr;
    b.cap = 0;
    bytes = std::max<size_t>(bytes, 256);
    if (cudaMallocAsync(&b.p, bytes, s) != cudaSuccess) {
        (void)cudaGetLastError();
        return BRM_ERR_ALLOC;
    }
    b.cap = bytes;
    return BRM_SUCCESS;
}

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// Offsets of every pair in the stacked operands: hp[i] and, in off, four
// arrays of n + 1 prefixes (A rows, A entries, B rows, B entries); the
// totals in ra, na, rb, nb, and cb = the largest B column count.  BRM_ERR_INVALID_VALUE for a
// malformed pair, BRM_ERR_CAPACITY when a total does not fit int32.
int batch_layout(int n, const brm_csr *A, const brm_csr *B, std::vector<brm::BatchPair> &hp,
                 std::vector<long long> &off, long long &ra, long long &na, long long &rb,
                 long long &nb, long long &cb)
{
    hp.assign((size_t)n, brm::BatchPair{});
    off.assign((size_t)(n + 1) * 4, 0);
    ra = na = rb = nb = cb = 0;
    for (int i = 0; i < n; i++) {
        const brm_csr &a = A[i], &b = B[i];
        if (a.M < 0 || a.N < 0 || b.M < 0 || b.N < 0 || a.nnz < 0 || b.nnz < 0 || a.N != b.M ||
            !a.rpt || !b.rpt || (a.nnz > 0 && (!a.col || !a.val)) ||
            (b.nnz > 0 && (!b.col || !b.val)))
            return BRM_ERR_INVALID_VALUE;
        brm::BatchPair &q = hp[(size_t)i];
        q.arpt = a.rpt;
        q.acol = a.col;
        q.aval = a.val;
        q.brpt = b.rpt;
        q.bcol = b.col;
        q.bval = b.val;
        q.M = a.M;
        q.K = a.N;
        q.N = b.N;
        q.nnzA = a.nnz;
        q.nnzB = b.nnz;
        q.row_a = ra;
        q.nnz_a = na;
        q.row_b = rb;
        q.nnz_b = nb;
        off[(size_t)i] = ra;
        off[(size_t)(n + 1) + i] = na;
        off[(size_t)2 * (n + 1) + i] = rb;
        off[(size_t)3 * (n + 1) + i] = nb;
        ra += a.M;
        na += a.nnz;
        rb += a.N;
        nb += b.nnz;
        cb = std::max<long long>(cb, b.N);
    }
    off[(size_t)n] = ra;
    off[(size_t)(n + 1) + n] = na;
    off[(size_t)2 * (n + 1) + n] = rb;
    off[(size_t)3 * (n + 1) + n] = nb;
    if (ra >= INT_MAX || na > INT_MAX || rb >= INT_MAX || nb > INT_MAX || cb > INT_MAX)
        return BRM_ERR_CAPACITY;  // the concatenation must fit int32 indices
    return BRM_SUCCESS;
}

// Gathers the pairs' columns (cols) and values into the stacked operands.
template <bool COLS>
void launch_entries_t(brm_dtype dtype, const brm::BatchPair *dp, int n, const long long *doff,
                      long long na, long long nb, int *A_col, void *A_val, int *B_col,
                      void *B_val, int grid, cudaStream_t s)
{
    if (dtype == BRM_F64) {
        brm::k_batch_entries<double, COLS><<<grid, 256, 0, s>>>(dp, n, doff + (n + 1), na, 0,
                                                                A_col, (double *)A_val);
        brm::count_launch();
        brm::k_batch_entries<double, COLS><<<grid, 256, 0, s>>>(dp, n, doff + 3 * (n + 1), nb, 1,
                                                                B_col, (double *)B_val);
        brm::count_launch();
    } else {
        brm::k_batch_entries<float, COLS><<<grid, 256, 0, s>>>(dp, n, doff + (n + 1), na, 0,
                                                               A_col, (float *)A_val);
        brm::count_launch();
        brm::k_batch_entries<float, COLS><<<grid, 256, 0, s>>>(dp, n, doff + 3 * (n + 1), nb, 1,
                                                               B_col, (float *)B_val);
        brm::count_launch();
    }
}

void launch_entries(brm_dtype dtype, const brm::BatchPair *dp, int n, const long long *doff,
                    long long na, long long nb, int *A_col, void *A_val, int *B_col, void *B_val,
                    int grid, cudaStream_t s, bool cols = true)
{
    if (cols)
        launch_entries_t<true>(dtype, dp, n, doff, na, nb, A_col, A_val, B_col, B_val, grid, s);
    else
        launch_entries_t<false>(dtype, dp, n, doff, na, nb, A_col, A_val, B_col, B_val, grid, s);
}

}  // namespace

extern "C" {

int brm_batch_precise(brm_context ctx, brm_dtype dtype, int n, const brm_csr *A, const brm_csr *B,
                      brm_batch *out)
{
    if (!ctx || !out || n < 0 || (n > 0 && (!A || !B)))
        return BRM_ERR_INVALID_VALUE;
    if (dtype != BRM_F64 && dtype != BRM_F32)
        return BRM_ERR_INVALID_VALUE;
    std::memset(out, 0, sizeof(*out));
    out->n = n;
    // offsets of every pair in the stacked operands
    std::vector<brm::BatchPair> hp;
    std::vector<long long> off;
    long long ra = 0, na = 0, rb = 0, nb = 0, cb = 0;
    {
        const int st = batch_layout(n, A, B, hp, off, ra, na, rb, nb, cb);
        if (st != BRM_SUCCESS)
            return st;
    }
    out->rows = ra;
    if (n == 0)
        return BRM_SUCCESS;
    cudaStream_t s = brm::context_stream(ctx);
    const size_t vb = dtype == BRM_F64 ? 8 : 4;
    // device scratch: pair table, offsets, A_bd, B_bd (freed at the end)
    Buf tab, abd, bbd;
    auto cleanup = [&]() {
        if (tab.p)
            cudaFreeAsync(tab.p, s);
        if (abd.p)
            cudaFreeAsync(abd.p, s);
        if (bbd.p)
            cudaFreeAsync(bbd.p, s);
    };
    const size_t b_pairs = a256(sizeof(brm::BatchPair) * (size_t)n);
    const size_t b_off = sizeof(long long) * off.size();
    int st = grow_buf(tab, b_pairs + a256(b_off) + sizeof(long long) * (size_t)(n + 1), s);
    const size_t a_rpt = a256(4 * (size_t)(ra + 1)), a_col = a256(4 * (size_t)std::max(na, 1LL));
    const size_t b_rpt = a256(4 * (size_t)(rb + 1)), b_col = a256(4 * (size_t)std::max(nb, 1LL));
    if (st == BRM_SUCCESS)
        st = grow_buf(abd, a_rpt + a_col + vb * (size_t)std::max(na, 1LL), s);
    if (st == BRM_SUCCESS)
        st = grow_buf(bbd, b_rpt + b_col + vb * (size_t)std::max(nb, 1LL), s);
    if (st != BRM_SUCCESS) {
        cleanup();
        return st;
    }
    brm::BatchPair *dp = (brm::BatchPair *)tab.p;
    long long *doff = (long long *)((char *)tab.p + b_pairs);
    long long *dfirst = (long long *)((char *)tab.p + b_pairs + a256(b_off));
    int *A_rpt = (int *)abd.p, *A_col = (int *)((char *)abd.p + a_rpt);
    void *A_val = (char *)abd.p + a_rpt + a_col;
    int *B_rpt = (int *)bbd.p, *B_col = (int *)((char *)bbd.p + b_rpt);
    void *B_val = (char *)bbd.p + b_rpt + b_col;
    cudaError_t e = cudaMemcpyAsync(dp, hp.data(), sizeof(brm::BatchPair) * (size_t)n,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(doff, off.data(), b_off, cudaMemcpyHostToDevice, s);
    const int sms = brm::context_num_sms(ctx);
    if (e == cudaSuccess) {
        const int g = std::max(sms, 1) * 16;
        brm::k_batch_rows<<<g, 256, 0, s>>>(dp, n, doff, ra, 0, A_rpt);
        brm::count_launch();
        brm::k_batch_rows<<<g, 256, 0, s>>>(dp, n, doff + 2 * (n + 1), rb, 1, B_rpt);
        brm::count_launch();
        launch_entries(dtype, dp, n, doff, na, nb, A_col, A_val, B_col, B_val, g, s);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        cleanup();
        return BRM_ERR_CUDA;
    }
    // one Precise call on the stacked operands
    brm_csr Abd{(int)ra, (int)rb, (int)na, A_rpt, A_col, A_val};
    brm_csr Bbd{(int)rb, (int)cb, (int)nb, B_rpt, B_col, B_val};
    int *crpt = nullptr, *ccol = nullptr;
    void *cval = nullptr;
    int cnnz = 0;
    st = brm_precise_device(ctx, dtype, &Abd, &Bbd, &crpt, &ccol, &cval, &cnnz, nullptr);
    if (st != BRM_SUCCESS) {
        cleanup();
        return st;
    }
    int *lrpt = nullptr;
    e = cudaMallocAsync((void **)&lrpt, sizeof(int) * (size_t)(ra + n), s);
    if (e == cudaSuccess) {
        const int g = std::max(sms, 1) * 16;
        brm::k_batch_first<<<g, 256, 0, s>>>(dp, n, (int)ra, crpt, dfirst);
        brm::count_launch();
        brm::k_batch_local_rpt<<<g, 256, 0, s>>>(n, doff, ra, crpt, dfirst, lrpt);
        brm::count_launch();
    }
    long long *hf = (long long *)std::malloc(sizeof(long long) * (size_t)(n + 1));
    long long *hr = (long long *)std::malloc(sizeof(long long) * (size_t)(n + 1));
    if (e == cudaSuccess)
        e = cudaGetLastError();
    if (hf && hr && e == cudaSuccess)
        e = cudaMemcpyAsync(hf, dfirst, sizeof(long long) * (size_t)(n + 1), cudaMemcpyDeviceToHost,
                            s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    cleanup();
    if (!hf || !hr || e != cudaSuccess) {
        (void)cudaGetLastError();
        std::free(hf);
        std::free(hr);
        brm_device_free(ctx, crpt);
        brm_device_free(ctx, ccol);
        brm_device_free(ctx, cval);
        brm_device_free(ctx, lrpt);
        return (!hf || !hr) ? BRM_ERR_ALLOC : BRM_ERR_CUDA;
    }
    std::memcpy(hr, off.data(), sizeof(long long) * (size_t)(n + 1));
    out->row_off = hr;
    out->nnz_off = hf;
    out->nnz = cnnz;
    out->crpt = crpt;
    out->ccol = ccol;
    out->cval = cval;
    out->rpt_local = lrpt;
    return BRM_SUCCESS;
}

int brm_batch_free(brm_context ctx, brm_batch *b)
{
    if (!b)
        return BRM_SUCCESS;
    int st = BRM_SUCCESS;
    if (b->crpt)
        st = brm_device_free(ctx, b->crpt);
    if (b->ccol && st == BRM_SUCCESS)
        st = brm_device_free(ctx, b->ccol);
    if (b->cval && st == BRM_SUCCESS)
        st = brm_device_free(ctx, b->cval);
    if (b->rpt_local && st == BRM_SUCCESS)
        st = brm_device_free(ctx, b->rpt_local);
    std::free(b->row_off);
    std::free(b->nnz_off);
    std::memset(b, 0, sizeof(*b));
    return st;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batch with a fixed structure replayed as a CUDA graph.  The stacked
// structure, the symbolic plan and C's row pointers are made once; the part
// that depends on the values (gathering every pair's current values into the
// stacked operands and the numeric phase) is captured once and replayed with
// one graph launch per recomputation.
// ---------------------------------------------------------------------------
struct brm_batch_graph_s {
    brm_context ctx = nullptr;     // private: its plan belongs to this batch
    cudaStream_t stream = nullptr;  // the private context's stream
    cudaStream_t cap = nullptr;     // capture stream
    brm_dtype dtype = BRM_F64;
    int n = 0;
    long long ra = 0, na = 0, rb = 0, nb = 0, cb = 0;
    void *mem = nullptr;            // pair table, offsets, first entries, A_bd, B_bd
    brm::BatchPair *dp = nullptr;
    long long *doff = nullptr, *dfirst = nullptr;
    brm_csr Abd{}, Bbd{};
    brm_batch out{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// Enqueues the value-dependent part on the private context's current
// stream: the pairs' current values into the stacked operands (their
// columns are fixed), then the numeric phase straight into C.
int batch_graph_values(brm_batch_graph g)
{
    cudaStream_t s = brm::context_stream(g->ctx);
    const int grid = std::max(brm::context_num_sms(g->ctx), 1) * 16;
    launch_entries(g->dtype, g->dp, g->n, g->doff, g->na, g->nb, (int *)g->Abd.col,
                   (void *)g->Abd.val, (int *)g->Bbd.col, (void *)g->Bbd.val, grid, s, false);
    const int st = brm::numeric_async(g->ctx, g->dtype, &g->Abd, &g->Bbd, g->out.crpt, g->out.ccol,
                                      g->out.cval);
    if (st != BRM_SUCCESS)
        return st;
    return cudaGetLastError() == cudaSuccess ? BRM_SUCCESS : BRM_ERR_CUDA;
}

}  // namespace

extern "C" {

int brm_batch_graph_destroy(brm_batch_graph g)
{
    if (!g)
        return BRM_SUCCESS;
    if (g->stream)
        cudaStreamSynchronize(g->stream);
    if (g->exec)
        cudaGraphExecDestroy(g->exec);
    if (g->graph)
        cudaGraphDestroy(g->graph);
    brm_batch_free(g->ctx, &g->out);
    if (g->mem)
        cudaFree(g->mem);
    if (g->ctx)
        brm_destroy(g->ctx);
    if (g->cap)
        cudaStreamDestroy(g->cap);
    if (g->stream)
        cudaStreamDestroy(g->stream);
    (void)cudaGetLastError();
    delete g;
    return BRM_SUCCESS;
}

int brm_batch_graph_create(brm_context ctx, brm_dtype dtype, int n, const brm_csr *A,
                           const brm_csr *B, brm_batch_graph *out_g, brm_batch *out)
{
    if (!ctx || !out_g || !out || n < 1 || !A || !B || (dtype != BRM_F64 && dtype != BRM_F32))
        return BRM_ERR_INVALID_VALUE;
    *out_g = nullptr;
    std::memset(out, 0, sizeof(*out));
    brm_batch_graph g = new (std::nothrow) brm_batch_graph_s();
    if (!g)
        return BRM_ERR_ALLOC;
    g->dtype = dtype;
    g->n = n;
    std::vector<brm::BatchPair> hp;
    std::vector<long long> off;
    int st = batch_layout(n, A, B, hp, off, g->ra, g->na, g->rb, g->nb, g->cb);
    brm_tuning tune;
    if (st == BRM_SUCCESS)
        st = brm_get_tuning(ctx, &tune);
    if (st == BRM_SUCCESS)
        st = brm_create(&g->ctx);
    if (st == BRM_SUCCESS)
        st = brm_set_tuning(g->ctx, &tune);
    if (st == BRM_SUCCESS &&
        (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess ||
         cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking) != cudaSuccess))
        st = BRM_ERR_CUDA;
    if (st == BRM_SUCCESS)
        st = brm_set_stream(g->ctx, g->stream);
    const size_t vb = dtype == BRM_F64 ? 8 : 4;
    const size_t b_pairs = a256(sizeof(brm::BatchPair) * (size_t)n);
    const size_t b_off = a256(sizeof(long long) * off.size());
    const size_t b_first = a256(sizeof(long long) * (size_t)(n + 1));
    const size_t a_rpt = a256(4 * (size_t)(g->ra + 1)), a_col = a256(4 * (size_t)std::max(g->na, 1LL));
    const size_t a_val = a256(vb * (size_t)std::max(g->na, 1LL));
    const size_t b_rpt = a256(4 * (size_t)(g->rb + 1)), b_col = a256(4 * (size_t)std::max(g->nb, 1LL));
    const size_t b_val = a256(vb * (size_t)std::max(g->nb, 1LL));
    if (st == BRM_SUCCESS &&
        cudaMalloc(&g->mem, b_pairs + b_off + b_first + a_rpt + a_col + a_val + b_rpt + b_col +
                                b_val) != cudaSuccess)
        st = BRM_ERR_ALLOC;
    if (st != BRM_SUCCESS) {
        (void)cudaGetLastError();
        brm_batch_graph_destroy(g);
        return st;
    }
    char *p = (char *)g->mem;
    g->dp = (brm::BatchPair *)p;
    g->doff = (long long *)(p += b_pairs);
    g->dfirst = (long long *)(p += b_off);
    int *A_rpt = (int *)(p += b_first);
    int *A_col = (int *)(p += a_rpt);
    void *A_val = (p += a_col);
    int *B_rpt = (int *)(p += a_val);
    int *B_col = (int *)(p += b_rpt);
    void *B_val = (p += b_col);
    g->Abd = brm_csr{(int)g->ra, (int)g->rb, (int)g->na, A_rpt, A_col, A_val};
    g->Bbd = brm_csr{(int)g->rb, (int)g->cb, (int)g->nb, B_rpt, B_col, B_val};
    cudaStream_t s = g->stream;
    const int grid = std::max(brm::context_num_sms(g->ctx), 1) * 16;
    cudaError_t e = cudaMemcpyAsync(g->dp, hp.data(), sizeof(brm::BatchPair) * (size_t)n,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g->doff, off.data(), sizeof(long long) * off.size(),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        brm::k_batch_rows<<<grid, 256, 0, s>>>(g->dp, n, g->doff, g->ra, 0, A_rpt);
        brm::count_launch();
        brm::k_batch_rows<<<grid, 256, 0, s>>>(g->dp, n, g->doff + 2 * (n + 1), g->rb, 1, B_rpt);
        brm::count_launch();
        launch_entries(dtype, g->dp, n, g->doff, g->na, g->nb, A_col, A_val, B_col, B_val, grid, s);
        e = cudaGetLastError();
    }
    // structure once: symbolic plan and C's row pointers, C's arrays
    int cnnz = 0;
    if (e == cudaSuccess &&
        cudaMallocAsync((void **)&g->out.crpt, 4 * (size_t)(g->ra + 1), s) != cudaSuccess)
        e = cudaErrorMemoryAllocation;
    st = e == cudaSuccess ? brm_symbolic(g->ctx, &g->Abd, &g->Bbd, g->out.crpt, &cnnz)
                          : BRM_ERR_CUDA;
    if (st == BRM_SUCCESS &&
        (cudaMallocAsync((void **)&g->out.ccol, 4 * (size_t)std::max(cnnz, 1), s) != cudaSuccess ||
         cudaMallocAsync(&g->out.cval, vb * (size_t)std::max(cnnz, 1), s) != cudaSuccess ||
         cudaMallocAsync((void **)&g->out.rpt_local, 4 * (size_t)(g->ra + n), s) != cudaSuccess))
        st = BRM_ERR_ALLOC;
    // first run, uncaptured: sizes every numeric buffer of the plan
    if (st == BRM_SUCCESS)
        st = batch_graph_values(g);
    if (st == BRM_SUCCESS) {
        brm::k_batch_first<<<grid, 256, 0, s>>>(g->dp, n, (int)g->ra, g->out.crpt, g->dfirst);
        brm::count_launch();
        brm::k_batch_local_rpt<<<grid, 256, 0, s>>>(n, g->doff, g->ra, g->out.crpt, g->dfirst,
                                                    g->out.rpt_local);
        brm::count_launch();
        st = brm::read_device_error(g->ctx);  // synchronises
    }
    g->out.n = n;
    g->out.rows = g->ra;
    g->out.nnz = cnnz;
    g->out.row_off = (long long *)std::malloc(sizeof(long long) * (size_t)(n + 1));
    g->out.nnz_off = (long long *)std::malloc(sizeof(long long) * (size_t)(n + 1));
    if (st == BRM_SUCCESS && (!g->out.row_off || !g->out.nnz_off))
        st = BRM_ERR_ALLOC;
    if (st == BRM_SUCCESS) {
        std::memcpy(g->out.row_off, off.data(), sizeof(long long) * (size_t)(n + 1));
        if (cudaMemcpy(g->out.nnz_off, g->dfirst, sizeof(long long) * (size_t)(n + 1),
                       cudaMemcpyDeviceToHost) != cudaSuccess)
            st = BRM_ERR_CUDA;
    }
    // capture the value-dependent part on a second stream
    if (st == BRM_SUCCESS) {
        brm_set_stream(g->ctx, g->cap);
        if (cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
            st = BRM_ERR_CUDA;
        } else {
            const int st2 = batch_graph_values(g);
            const cudaError_t e2 = cudaStreamEndCapture(g->cap, &g->graph);
            st = st2 != BRM_SUCCESS ? st2 : (e2 == cudaSuccess ? BRM_SUCCESS : BRM_ERR_CUDA);
        }
        brm_set_stream(g->ctx, g->stream);
        if (st == BRM_SUCCESS && cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess)
            st = BRM_ERR_CUDA;
    }
    if (st != BRM_SUCCESS) {
        (void)cudaGetLastError();
        brm_batch_graph_destroy(g);
        std::memset(out, 0, sizeof(*out));
        return st;
    }
    *out = g->out;
    *out_g = g;
    return BRM_SUCCESS;
}

int brm_batch_graph_launch(brm_batch_graph g, void *stream)
{
    if (!g || !g->exec)
        return BRM_ERR_INVALID_VALUE;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaGraphLaunch(g->exec, s) != cudaSuccess) {
        (void)cudaGetLastError();
        return BRM_ERR_CUDA;
    }
    // the numeric phase's error word, read on the launch stream
    brm_set_stream(g->ctx, s);
    const int st = brm::read_device_error(g->ctx);
    brm_set_stream(g->ctx, g->stream);
    return st;
}

}  // extern "C"
