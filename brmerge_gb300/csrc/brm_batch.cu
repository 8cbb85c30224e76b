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
#include <cmath>
#include <cstdint>
#include <type_traits>
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

// The batch in flight, in device memory next to its pair table: the
// kernels read the sizes from here, so a captured graph serves any batch.
// Offsets are four arrays of `stride` entries (stride >= n + 1): A rows, A
// entries, B rows, B entries, each the prefix over the pairs.
struct BatchDims {
    long long n;
    long long rows_a, nnz_a, rows_b, nnz_b;
};

// Row pointers of A_bd (which = 0) or B_bd (which = 1) for rows [0, cap]:
// rows past the batch are empty (a captured pipeline pads the stacked
// operands to its capacity).
__global__ void __launch_bounds__(256) k_batch_rows(const BatchDims *dims, const BatchPair *pairs,
                                                    const long long *off, int stride, long long cap,
                                                    int which, int *rpt)
{
    const int n = (int)dims->n;
    const long long rows = which == 0 ? dims->rows_a : dims->rows_b;
    const long long tot = which == 0 ? dims->nnz_a : dims->nnz_b;
    const long long *row_off = off + (size_t)(which == 0 ? 0 : 2) * stride;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r <= cap;
         r += (long long)gridDim.x * blockDim.x) {
        if (r >= rows) {
            rpt[r] = (int)tot;
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
__global__ void __launch_bounds__(256) k_batch_entries(const BatchDims *dims,
                                                       const BatchPair *pairs,
                                                       const long long *off, int stride,
                                                       int which, int *col, T *val)
{
    const int n = (int)dims->n;
    const long long nnz = which == 0 ? dims->nnz_a : dims->nnz_b;
    const long long *nnz_off = off + (size_t)(which == 0 ? 1 : 3) * stride;
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
__global__ void __launch_bounds__(256) k_batch_first(const BatchDims *dims, const BatchPair *pairs,
                                                     const int *crpt, long long *nnz_first)
{
    const long long n = dims->n;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
         i += (long long)gridDim.x * blockDim.x)
        nnz_first[i] = crpt[i < n ? pairs[i].row_a : dims->rows_a];
}

// Each pair's own row pointers (starting at 0), pair i at out[row_off[i] +
// i .. row_off[i+1] + i].
__global__ void __launch_bounds__(256) k_batch_local_rpt(const BatchDims *dims,
                                                         const long long *off, const int *crpt,
                                                         const long long *first, int *out)
{
    const int n = (int)dims->n;
    const long long rows = dims->rows_a;
    const long long *row_off = off;
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

#define BRM_STATUS_TRY(call)   \
    do {                       \
        const int s_ = (call); \
        if (s_ != BRM_SUCCESS) \
            return s_;         \
    } while (0)

// The batch's table in device memory (and its host image, same layout):
// dims, the pair table and the four offset arrays, contiguous so that one
// copy uploads them, then each pair's first entry in C.  Sized for at most
// max_pairs pairs; every offset array has stride = max_pairs + 1 entries.
struct BatchTable {
    brm::BatchDims *dims = nullptr;
    brm::BatchPair *pairs = nullptr;
    long long *off = nullptr;
    long long *first = nullptr;
    int stride = 1;
    size_t upload = 0;  // bytes of dims + pairs + offsets
    size_t bytes = 0;   // the whole table
};

BatchTable table_layout(void *base, int max_pairs)
{
    BatchTable t;
    t.stride = max_pairs + 1;
    const size_t b_dims = a256(sizeof(brm::BatchDims));
    const size_t b_pairs = a256(sizeof(brm::BatchPair) * (size_t)std::max(max_pairs, 1));
    const size_t b_off = a256(sizeof(long long) * 4 * (size_t)t.stride);
    const size_t b_first = a256(sizeof(long long) * (size_t)t.stride);
    unsigned char *p = (unsigned char *)base;
    t.dims = (brm::BatchDims *)p;
    t.pairs = (brm::BatchPair *)(p + b_dims);
    t.off = (long long *)(p + b_dims + b_pairs);
    t.first = (long long *)(p + b_dims + b_pairs + b_off);
    t.upload = b_dims + b_pairs + b_off;
    t.bytes = t.upload + b_first;
    return t;
}

// Offsets of every pair in the stacked operands, written into the host image
// of a table: dims (the totals), the pair table and the four prefix arrays
// (A rows, A entries, B rows, B entries); cb = the largest B column count.
// BRM_ERR_INVALID_VALUE for a malformed pair, BRM_ERR_CAPACITY when a total
// does not fit int32.
int batch_layout(int n, const brm_csr *A, const brm_csr *B, const BatchTable &img, long long &cb)
{
    brm::BatchDims &d = *img.dims;
    d = brm::BatchDims{n, 0, 0, 0, 0};
    long long *off = img.off;
    const int st = img.stride;
    cb = 0;
    for (int i = 0; i < n; i++) {
        const brm_csr &a = A[i], &b = B[i];
        if (a.M < 0 || a.N < 0 || b.M < 0 || b.N < 0 || a.nnz < 0 || b.nnz < 0 || a.N != b.M ||
            !a.rpt || !b.rpt || (a.nnz > 0 && (!a.col || !a.val)) ||
            (b.nnz > 0 && (!b.col || !b.val)))
            return BRM_ERR_INVALID_VALUE;
        brm::BatchPair &q = img.pairs[i];
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
        q.row_a = d.rows_a;
        q.nnz_a = d.nnz_a;
        q.row_b = d.rows_b;
        q.nnz_b = d.nnz_b;
        off[i] = d.rows_a;
        off[st + i] = d.nnz_a;
        off[2 * st + i] = d.rows_b;
        off[3 * st + i] = d.nnz_b;
        d.rows_a += a.M;
        d.nnz_a += a.nnz;
        d.rows_b += a.N;
        d.nnz_b += b.nnz;
        cb = std::max<long long>(cb, b.N);
    }
    off[n] = d.rows_a;
    off[st + n] = d.nnz_a;
    off[2 * st + n] = d.rows_b;
    off[3 * st + n] = d.nnz_b;
    if (d.rows_a >= INT_MAX || d.nnz_a > INT_MAX || d.rows_b >= INT_MAX || d.nnz_b > INT_MAX ||
        cb > INT_MAX)
        return BRM_ERR_CAPACITY;  // the concatenation must fit int32 indices
    return BRM_SUCCESS;
}

// The stacked operands from the pairs: row pointers of A_bd and B_bd for
// rows [0, cap_a] and [0, cap_b] (rows past the batch empty), and their
// columns (cols) and values.
void launch_stack(brm_dtype dtype, const BatchTable &t, long long cap_a, long long cap_b,
                  const brm_csr &Abd, const brm_csr &Bbd, int grid, cudaStream_t s, bool cols)
{
    if (cols) {
        brm::k_batch_rows<<<grid, 256, 0, s>>>(t.dims, t.pairs, t.off, t.stride, cap_a, 0,
                                               (int *)Abd.rpt);
        brm::count_launch();
        brm::k_batch_rows<<<grid, 256, 0, s>>>(t.dims, t.pairs, t.off, t.stride, cap_b, 1,
                                               (int *)Bbd.rpt);
        brm::count_launch();
    }
    auto go = [&](auto tag, auto ctag) {
        using T = decltype(tag);
        constexpr bool C = decltype(ctag)::value;
        brm::k_batch_entries<T, C><<<grid, 256, 0, s>>>(t.dims, t.pairs, t.off, t.stride, 0,
                                                        (int *)Abd.col, (T *)Abd.val);
        brm::count_launch();
        brm::k_batch_entries<T, C><<<grid, 256, 0, s>>>(t.dims, t.pairs, t.off, t.stride, 1,
                                                        (int *)Bbd.col, (T *)Bbd.val);
        brm::count_launch();
    };
    if (dtype == BRM_F64) {
        if (cols)
            go(double(), std::true_type());
        else
            go(double(), std::false_type());
    } else {
        if (cols)
            go(float(), std::true_type());
        else
            go(float(), std::false_type());
    }
}

// Each pair's first entry in C and its own row pointers (rpt_local).
void launch_finish(const BatchTable &t, const int *crpt, int *lrpt, int grid, cudaStream_t s)
{
    brm::k_batch_first<<<grid, 256, 0, s>>>(t.dims, t.pairs, crpt, t.first);
    brm::count_launch();
    brm::k_batch_local_rpt<<<grid, 256, 0, s>>>(t.dims, t.off, crpt, t.first, lrpt);
    brm::count_launch();
}

// A host image of a batch table (pageable; copied in one cudaMemcpyAsync
// that the call synchronises before the image is released).
struct HostTable {
    std::vector<unsigned char> mem;
    BatchTable t;
    explicit HostTable(int max_pairs)
    {
        t = table_layout(nullptr, max_pairs);
        mem.assign(t.bytes + 256, 0);
        unsigned char *base = (unsigned char *)(((uintptr_t)mem.data() + 255) & ~uintptr_t(255));
        t = table_layout(base, max_pairs);
    }
};

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
    HostTable h(n);
    long long cb = 0;
    {
        const int st = batch_layout(n, A, B, h.t, cb);
        if (st != BRM_SUCCESS)
            return st;
    }
    const brm::BatchDims dm = *h.t.dims;
    const long long ra = dm.rows_a, na = dm.nnz_a, rb = dm.rows_b, nb = dm.nnz_b;
    out->rows = ra;
    if (n == 0)
        return BRM_SUCCESS;
    cudaStream_t s = brm::context_stream(ctx);
    const size_t vb = dtype == BRM_F64 ? 8 : 4;
    // device scratch: the table, A_bd, B_bd (freed at the end)
    Buf tab, abd, bbd;
    auto cleanup = [&]() {
        if (tab.p)
            cudaFreeAsync(tab.p, s);
        if (abd.p)
            cudaFreeAsync(abd.p, s);
        if (bbd.p)
            cudaFreeAsync(bbd.p, s);
    };
    int st = grow_buf(tab, h.t.bytes, s);
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
    const BatchTable t = table_layout(tab.p, n);
    int *A_rpt = (int *)abd.p, *A_col = (int *)((char *)abd.p + a_rpt);
    void *A_val = (char *)abd.p + a_rpt + a_col;
    int *B_rpt = (int *)bbd.p, *B_col = (int *)((char *)bbd.p + b_rpt);
    void *B_val = (char *)bbd.p + b_rpt + b_col;
    brm_csr Abd{(int)ra, (int)rb, (int)na, A_rpt, A_col, A_val};
    brm_csr Bbd{(int)rb, (int)cb, (int)nb, B_rpt, B_col, B_val};
    cudaError_t e = cudaMemcpyAsync(t.dims, h.t.dims, t.upload, cudaMemcpyHostToDevice, s);
    const int sms = brm::context_num_sms(ctx);
    const int g = std::max(sms, 1) * 16;
    if (e == cudaSuccess) {
        launch_stack(dtype, t, ra, rb, Abd, Bbd, g, s, true);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        cleanup();
        return BRM_ERR_CUDA;
    }
    // one Precise call on the stacked operands
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
        launch_finish(t, crpt, lrpt, g, s);
        e = cudaGetLastError();
    }
    long long *hf = (long long *)std::malloc(sizeof(long long) * (size_t)(n + 1));
    long long *hr = (long long *)std::malloc(sizeof(long long) * (size_t)(n + 1));
    if (hf && hr && e == cudaSuccess)
        e = cudaMemcpyAsync(hf, t.first, sizeof(long long) * (size_t)(n + 1),
                            cudaMemcpyDeviceToHost, s);
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
    std::memcpy(hr, h.t.off, sizeof(long long) * (size_t)(n + 1));
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
    void *mem = nullptr;            // the batch table, A_bd, B_bd
    BatchTable t;
    brm_csr Abd{}, Bbd{};
    brm_batch out{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;          // kernels in the graph (counted at each launch)
};

namespace {

// Enqueues the value-dependent part on the private context's current
// stream: the pairs' current values into the stacked operands (their
// columns are fixed), then the numeric phase straight into C.
int batch_graph_values(brm_batch_graph g)
{
    cudaStream_t s = brm::context_stream(g->ctx);
    const int grid = std::max(brm::context_num_sms(g->ctx), 1) * 16;
    launch_stack(g->dtype, g->t, g->Abd.M, g->Bbd.M, g->Abd, g->Bbd, grid, s, false);
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
    HostTable h(n);
    long long cb = 0;
    int st = batch_layout(n, A, B, h.t, cb);
    const brm::BatchDims dm = *h.t.dims;
    const long long ra = dm.rows_a, na = dm.nnz_a, rb = dm.rows_b, nb = dm.nnz_b;
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
    const size_t b_tab = a256(h.t.bytes);
    const size_t a_rpt = a256(4 * (size_t)(ra + 1)), a_col = a256(4 * (size_t)std::max(na, 1LL));
    const size_t a_val = a256(vb * (size_t)std::max(na, 1LL));
    const size_t b_rpt = a256(4 * (size_t)(rb + 1)), b_col = a256(4 * (size_t)std::max(nb, 1LL));
    const size_t b_val = a256(vb * (size_t)std::max(nb, 1LL));
    if (st == BRM_SUCCESS &&
        cudaMalloc(&g->mem, b_tab + a_rpt + a_col + a_val + b_rpt + b_col + b_val) != cudaSuccess)
        st = BRM_ERR_ALLOC;
    if (st != BRM_SUCCESS) {
        (void)cudaGetLastError();
        brm_batch_graph_destroy(g);
        return st;
    }
    char *p = (char *)g->mem;
    g->t = table_layout(p, n);
    int *A_rpt = (int *)(p += b_tab);
    int *A_col = (int *)(p += a_rpt);
    void *A_val = (p += a_col);
    int *B_rpt = (int *)(p += a_val);
    int *B_col = (int *)(p += b_rpt);
    void *B_val = (p += b_col);
    g->Abd = brm_csr{(int)ra, (int)rb, (int)na, A_rpt, A_col, A_val};
    g->Bbd = brm_csr{(int)rb, (int)cb, (int)nb, B_rpt, B_col, B_val};
    cudaStream_t s = g->stream;
    const int grid = std::max(brm::context_num_sms(g->ctx), 1) * 16;
    cudaError_t e = cudaMemcpyAsync(g->t.dims, h.t.dims, g->t.upload, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        launch_stack(dtype, g->t, ra, rb, g->Abd, g->Bbd, grid, s, true);
        e = cudaGetLastError();
    }
    // structure once: symbolic plan and C's row pointers, C's arrays
    int cnnz = 0;
    if (e == cudaSuccess &&
        cudaMallocAsync((void **)&g->out.crpt, 4 * (size_t)(ra + 1), s) != cudaSuccess)
        e = cudaErrorMemoryAllocation;
    st = e == cudaSuccess ? brm_symbolic(g->ctx, &g->Abd, &g->Bbd, g->out.crpt, &cnnz)
                          : BRM_ERR_CUDA;
    if (st == BRM_SUCCESS &&
        (cudaMallocAsync((void **)&g->out.ccol, 4 * (size_t)std::max(cnnz, 1), s) != cudaSuccess ||
         cudaMallocAsync(&g->out.cval, vb * (size_t)std::max(cnnz, 1), s) != cudaSuccess ||
         cudaMallocAsync((void **)&g->out.rpt_local, 4 * (size_t)(ra + n), s) != cudaSuccess))
        st = BRM_ERR_ALLOC;
    // first run, uncaptured: sizes every numeric buffer of the plan
    if (st == BRM_SUCCESS)
        st = batch_graph_values(g);
    if (st == BRM_SUCCESS) {
        launch_finish(g->t, g->out.crpt, g->out.rpt_local, grid, s);
        st = brm::read_device_error(g->ctx);  // synchronises
    }
    g->out.n = n;
    g->out.rows = ra;
    g->out.nnz = cnnz;
    g->out.row_off = (long long *)std::malloc(sizeof(long long) * (size_t)(n + 1));
    g->out.nnz_off = (long long *)std::malloc(sizeof(long long) * (size_t)(n + 1));
    if (st == BRM_SUCCESS && (!g->out.row_off || !g->out.nnz_off))
        st = BRM_ERR_ALLOC;
    if (st == BRM_SUCCESS) {
        std::memcpy(g->out.row_off, h.t.off, sizeof(long long) * (size_t)(n + 1));
        if (cudaMemcpy(g->out.nnz_off, g->t.first, sizeof(long long) * (size_t)(n + 1),
                       cudaMemcpyDeviceToHost) != cudaSuccess)
            st = BRM_ERR_CUDA;
    }
    // capture the value-dependent part on a second stream
    if (st == BRM_SUCCESS) {
        brm_set_stream(g->ctx, g->cap);
        if (cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
            st = BRM_ERR_CUDA;
        } else {
            const long long k0 = brm::launches_so_far();
            const int st2 = batch_graph_values(g);
            g->kernels = brm::launches_so_far() - k0;
            brm::count_launches(-g->kernels);  // captured, not launched
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
    brm::count_launches(g->kernels);
    // the numeric phase's error word, read on the launch stream
    brm_set_stream(g->ctx, s);
    const int st = brm::read_device_error(g->ctx);
    brm_set_stream(g->ctx, g->stream);
    return st;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batch pipeline: a whole brm_batch_precise (stacking, planning, numeric
// phase, per-pair offsets) captured once as a CUDA graph with fixed
// capacities, then launched once per new batch, whatever its structure.  The
// stacked operands are padded to the capacities (rows past the batch are
// empty), the kernels read the batch's sizes from its table in device memory,
// and admission kernels stop the pipeline on the device when a batch's
// products, segments, split table or spill scratch exceed the capacities.
// ---------------------------------------------------------------------------
struct brm_batch_pipe_s {
    brm_context ctx = nullptr;      // private: plan buffers grown to the capacities
    cudaStream_t stream = nullptr;  // capture stream (the private context's stream)
    brm_dtype dtype = BRM_F64;
    brm_batch_caps caps{};
    brm::PipeCaps pc{};
    void *mem = nullptr;            // device: table, A_bd, B_bd, C, rpt_local
    BatchTable t;                   // device table
    void *host = nullptr;           // page-locked: table image, counters, first entries
    BatchTable ht;                  // host image of the table (uploaded by the graph)
    brm::Counters *hcnt = nullptr;  // counters copied back by the graph
    long long *hfirst = nullptr;    // first entries copied back by the graph
    brm_csr Abd{}, Bbd{};
    int *crpt = nullptr, *ccol = nullptr, *lrpt = nullptr;
    void *cval = nullptr;
    long long *row_off = nullptr, *nnz_off = nullptr;  // host, pairs + 1
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;
};

extern "C" {

int brm_batch_caps_for(brm_context ctx, brm_dtype dtype, int n, const brm_csr *A,
                       const brm_csr *B, double headroom, brm_batch_caps *caps)
{
    if (!ctx || !caps || n < 1 || !A || !B || !(headroom >= 1.0) || headroom > 1e3 ||
        (dtype != BRM_F64 && dtype != BRM_F32))
        return BRM_ERR_INVALID_VALUE;
    HostTable h(n);
    long long cb = 0;
    BRM_STATUS_TRY(batch_layout(n, A, B, h.t, cb));
    brm_batch b;
    BRM_STATUS_TRY(brm_batch_precise(ctx, dtype, n, A, B, &b));  // plans the sample
    const brm::Counters c = brm::last_plan_counters(ctx);
    brm_batch_free(ctx, &b);
    const brm::BatchDims d = *h.t.dims;
    auto up = [&](long long x, long long lo) {
        const double v = std::ceil((double)x * headroom);
        return std::max<long long>(lo, v > 2e18 ? (long long)2e18 : (long long)v);
    };
    caps->pairs = (int)std::min<long long>(up(n, 1), INT_MAX - 1);
    caps->rows = std::min<long long>(up(d.rows_a, 1), INT_MAX - 1);
    caps->nnz_a = std::min<long long>(up(d.nnz_a, 1), INT_MAX);
    caps->b_rows = std::min<long long>(up(d.rows_b, 1), INT_MAX - 1);
    caps->nnz_b = std::min<long long>(up(d.nnz_b, 1), INT_MAX);
    caps->cols = (int)std::min<long long>(up(cb, 1), INT_MAX);
    caps->products = std::min<long long>(up((long long)c.total_flop, 1), INT_MAX);
    caps->seg_slots = up((long long)c.seg_cap, 0) + 1024;
    caps->table = up((long long)c.table_cap, 0) + 65536;
    caps->spill_bytes = up((long long)c.spill_bytes, 64ll << 20);
    return BRM_SUCCESS;
}

int brm_batch_pipe_destroy(brm_batch_pipe p)
{
    if (!p)
        return BRM_SUCCESS;
    if (p->stream)
        cudaStreamSynchronize(p->stream);
    if (p->exec)
        cudaGraphExecDestroy(p->exec);
    if (p->graph)
        cudaGraphDestroy(p->graph);
    if (p->mem)
        cudaFree(p->mem);
    if (p->host)
        cudaFreeHost(p->host);
    if (p->ctx)
        brm_destroy(p->ctx);
    if (p->stream)
        cudaStreamDestroy(p->stream);
    std::free(p->row_off);
    std::free(p->nnz_off);
    (void)cudaGetLastError();
    delete p;
    return BRM_SUCCESS;
}

int brm_batch_pipe_create(brm_context ctx, brm_dtype dtype, const brm_batch_caps *caps,
                          brm_batch_pipe *out)
{
    if (!ctx || !caps || !out || (dtype != BRM_F64 && dtype != BRM_F32))
        return BRM_ERR_INVALID_VALUE;
    *out = nullptr;
    const brm_batch_caps &c = *caps;
    if (c.pairs < 1 || c.rows < 1 || c.nnz_a < 0 || c.b_rows < 1 || c.nnz_b < 0 || c.cols < 1 ||
        c.products < 0 || c.seg_slots < 0 || c.table < 0 || c.spill_bytes < 0)
        return BRM_ERR_INVALID_VALUE;
    if (c.rows >= INT_MAX || c.nnz_a > INT_MAX || c.b_rows >= INT_MAX || c.nnz_b > INT_MAX ||
        c.products > INT_MAX || c.pairs >= INT_MAX)
        return BRM_ERR_CAPACITY;  // int32 CSR: nnz of all C_i together is at most the products
    brm_batch_pipe p = new (std::nothrow) brm_batch_pipe_s();
    if (!p)
        return BRM_ERR_ALLOC;
    p->dtype = dtype;
    p->caps = c;
    p->pc = brm::PipeCaps{c.rows, c.nnz_a, c.b_rows, c.nnz_b, (long long)c.cols, c.products,
                          c.seg_slots, c.table, c.spill_bytes};
    brm_tuning tune;
    int st = brm_get_tuning(ctx, &tune);
    if (st == BRM_SUCCESS)
        st = brm_create(&p->ctx);
    if (st == BRM_SUCCESS)
        st = brm_set_tuning(p->ctx, &tune);
    if (st == BRM_SUCCESS &&
        cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess)
        st = BRM_ERR_CUDA;
    if (st == BRM_SUCCESS)
        st = brm_set_stream(p->ctx, p->stream);
    // device memory: table, A_bd, B_bd, C (crpt, ccol, cval), rpt_local
    const size_t vb = dtype == BRM_F64 ? 8 : 4;
    const BatchTable tl = table_layout(nullptr, c.pairs);
    const size_t b_tab = a256(tl.bytes);
    const size_t a_rpt = a256(4 * (size_t)(c.rows + 1)), a_col = a256(4 * (size_t)std::max(c.nnz_a, 1LL));
    const size_t a_val = a256(vb * (size_t)std::max(c.nnz_a, 1LL));
    const size_t b_rpt = a256(4 * (size_t)(c.b_rows + 1)), b_col = a256(4 * (size_t)std::max(c.nnz_b, 1LL));
    const size_t b_val = a256(vb * (size_t)std::max(c.nnz_b, 1LL));
    const size_t c_rpt = a256(4 * (size_t)(c.rows + 1)), c_col = a256(4 * (size_t)std::max(c.products, 1LL));
    const size_t c_val = a256(vb * (size_t)std::max(c.products, 1LL));
    const size_t l_rpt = a256(4 * (size_t)(c.rows + c.pairs));
    if (st == BRM_SUCCESS &&
        cudaMalloc(&p->mem, b_tab + a_rpt + a_col + a_val + b_rpt + b_col + b_val + c_rpt + c_col +
                                c_val + l_rpt) != cudaSuccess)
        st = BRM_ERR_ALLOC;
    const size_t h_cnt = a256(sizeof(brm::Counters));
    const size_t h_first = a256(sizeof(long long) * (size_t)tl.stride);
    if (st == BRM_SUCCESS && cudaMallocHost(&p->host, b_tab + h_cnt + h_first) != cudaSuccess)
        st = BRM_ERR_ALLOC;
    p->row_off = (long long *)std::malloc(sizeof(long long) * ((size_t)c.pairs + 1));
    p->nnz_off = (long long *)std::malloc(sizeof(long long) * ((size_t)c.pairs + 1));
    if (st == BRM_SUCCESS && (!p->row_off || !p->nnz_off))
        st = BRM_ERR_ALLOC;
    if (st == BRM_SUCCESS)
        st = brm::reserve_pipe(p->ctx, dtype, p->pc);
    if (st != BRM_SUCCESS) {
        (void)cudaGetLastError();
        brm_batch_pipe_destroy(p);
        return st;
    }
    char *q = (char *)p->mem;
    p->t = table_layout(q, c.pairs);
    int *A_rpt = (int *)(q += b_tab);
    int *A_col = (int *)(q += a_rpt);
    void *A_val = (q += a_col);
    int *B_rpt = (int *)(q += a_val);
    int *B_col = (int *)(q += b_rpt);
    void *B_val = (q += b_col);
    p->crpt = (int *)(q += b_val);
    p->ccol = (int *)(q += c_rpt);
    p->cval = (q += c_col);
    p->lrpt = (int *)(q += c_val);
    p->Abd = brm_csr{(int)c.rows, (int)c.b_rows, (int)c.nnz_a, A_rpt, A_col, A_val};
    p->Bbd = brm_csr{(int)c.b_rows, c.cols, (int)c.nnz_b, B_rpt, B_col, B_val};
    p->ht = table_layout(p->host, c.pairs);
    p->hcnt = (brm::Counters *)((char *)p->host + b_tab);
    p->hfirst = (long long *)((char *)p->host + b_tab + h_cnt);
    std::memset(p->host, 0, b_tab + h_cnt + h_first);
    // capture: upload the table, stack, Precise, per-pair offsets, results back
    cudaStream_t s = p->stream;
    const int grid = std::max(brm::context_num_sms(p->ctx), 1) * 16;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        (void)cudaGetLastError();
        brm_batch_pipe_destroy(p);
        return BRM_ERR_CUDA;
    }
    const long long k0 = brm::launches_so_far();
    cudaError_t e = cudaMemcpyAsync(p->t.dims, p->ht.dims, p->t.upload, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        launch_stack(dtype, p->t, c.rows, c.b_rows, p->Abd, p->Bbd, grid, s, true);
        st = brm::precise_pipe(p->ctx, dtype, &p->Abd, &p->Bbd, p->crpt, p->ccol, p->cval, p->pc);
    }
    if (e == cudaSuccess && st == BRM_SUCCESS) {
        launch_finish(p->t, p->crpt, p->lrpt, grid, s);
        e = cudaMemcpyAsync(p->hcnt, brm::context_counters(p->ctx), sizeof(brm::Counters),
                            cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess && st == BRM_SUCCESS)
        e = cudaMemcpyAsync(p->hfirst, p->t.first, sizeof(long long) * (size_t)p->t.stride,
                            cudaMemcpyDeviceToHost, s);
    p->kernels = brm::launches_so_far() - k0;
    brm::count_launches(-p->kernels);  // captured, not launched
    const cudaError_t e2 = cudaStreamEndCapture(s, &p->graph);
    if (st == BRM_SUCCESS && (e != cudaSuccess || e2 != cudaSuccess))
        st = BRM_ERR_CUDA;
    if (st == BRM_SUCCESS && cudaGraphInstantiate(&p->exec, p->graph, 0) != cudaSuccess)
        st = BRM_ERR_CUDA;
    if (st != BRM_SUCCESS) {
        (void)cudaGetLastError();
        brm_batch_pipe_destroy(p);
        return st;
    }
    *out = p;
    return BRM_SUCCESS;
}

int brm_batch_pipe_caps(brm_batch_pipe p, brm_batch_caps *caps)
{
    if (!p || !caps)
        return BRM_ERR_INVALID_VALUE;
    *caps = p->caps;
    return BRM_SUCCESS;
}

int brm_batch_pipe_run(brm_batch_pipe p, int n, const brm_csr *A, const brm_csr *B, void *stream,
                       brm_batch *out)
{
    if (!p || !out || n < 1 || !A || !B)
        return BRM_ERR_INVALID_VALUE;
    std::memset(out, 0, sizeof(*out));
    if (n > p->caps.pairs)
        return BRM_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    // the previous launch of this pipe has finished (every run synchronises),
    // so the page-locked table image is free to overwrite
    long long cb = 0;
    BRM_STATUS_TRY(batch_layout(n, A, B, p->ht, cb));
    const brm::BatchDims d = *p->ht.dims;
    if (d.rows_a > p->caps.rows || d.nnz_a > p->caps.nnz_a || d.rows_b > p->caps.b_rows ||
        d.nnz_b > p->caps.nnz_b || cb > p->caps.cols)
        return BRM_ERR_CAPACITY;
    if (cudaGraphLaunch(p->exec, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
        (void)cudaGetLastError();
        return BRM_ERR_CUDA;
    }
    brm::count_launches(p->kernels);
    if (p->hcnt->abort)
        return BRM_ERR_CAPACITY;
    BRM_STATUS_TRY(brm::device_status(p->hcnt->err));
    if (p->hcnt->cnnz > INT_MAX)
        return BRM_ERR_OVERFLOW;
    std::memcpy(p->row_off, p->ht.off, sizeof(long long) * (size_t)(n + 1));
    std::memcpy(p->nnz_off, p->hfirst, sizeof(long long) * (size_t)(n + 1));
    out->n = n;
    out->rows = d.rows_a;
    out->nnz = p->hcnt->cnnz;
    out->row_off = p->row_off;
    out->nnz_off = p->nnz_off;
    out->crpt = p->crpt;
    out->ccol = p->ccol;
    out->cval = p->cval;
    out->rpt_local = p->lrpt;
    return BRM_SUCCESS;
}

}  // extern "C"
