// brm_noalloc.cu -- product count that allocates no memory.
//
// Some callers may not allocate device memory at the moment they need an
// answer: an admission controller deciding whether a request fits before it
// reserves anything, code running while the caching allocator is locked or
// its pool is exhausted, or a host thread that must not trigger the implicit
// synchronisation of cudaMalloc/cudaFree.  brm_compute_flop_noalloc gives
// them the per-row intermediate-product counts of A*B (the quantity the
// reference's compute_flop returns, BRMerge-SpGEMM/inc/spgemm.h:8-29) without
// any allocation: the reduction scratch is the fixed array below, and the
// caller provides the only output buffer.
//
// The array lives in every GPU that loads this library until the process
// exits (kNoAllocMaxBlocks + 2 words = 512 KB + 16 bytes).  All calls share
// it, so calls whose work overlaps on the GPU (different streams, different
// host threads) race on it; serialise them.  Each call clears what must start
// at zero (the error word) and overwrites the rest.
//
// The device address of the array is looked up once per device and kept for
// the life of the process.  A cudaDeviceReset (or anything else that tears
// down and recreates the device's primary context) reloads this library's
// device code at a possibly different address, so the kept address is stale
// afterwards: do not use this entry point after resetting a device.
#include <climits>
#include <mutex>

#include "brm_common.cuh"
#include "brmerge.h"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocRowsPerBlock = 64;  // 8 warps x 8 rows
constexpr int kNoAllocMaxBlocks = 65536;
constexpr long long kNoAllocMaxRows = (long long)kNoAllocMaxBlocks * kNoAllocRowsPerBlock;
constexpr int kMaxDevices = 64;

// [0, kNoAllocMaxBlocks): per-block partial sums; [kNoAllocMaxBlocks]: total;
// [kNoAllocMaxBlocks + 1]: error word (kNaBadInput | kNaRowOverflow).
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocMaxBlocks + 2];

// Host-side stand-ins are not device addresses: the device address of the
// array is looked up once per device with that device current.
constexpr unsigned long long kNaBadInput = 1;     // A.rpt, A.col or B.rpt not valid CSR
constexpr unsigned long long kNaRowOverflow = 2;  // a row's count above INT_MAX

std::mutex g_noalloc_mu;
unsigned long long *g_noalloc_dev[kMaxDevices] = {};

// Per-row products (warp per row) and one partial sum per block, written to
// the block's own scratch slot (no atomics: the total is deterministic).
__global__ void __launch_bounds__(kNoAllocThreads)
    k_flop_noalloc(brm_csr A, brm_csr B, int *row_flop, unsigned long long *scratch)
{
    __shared__ unsigned long long s_part[kNoAllocThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int M = A.M, K = B.M;
    const int rows_per_warp = kNoAllocRowsPerBlock / (kNoAllocThreads / 32);
    unsigned long long wsum = 0;
    bool bad = false, big = false;
    for (int r = 0; r < rows_per_warp; r++) {
        const int row = blockIdx.x * kNoAllocRowsPerBlock + w * rows_per_warp + r;
        if (row >= M)
            break;
        int a0 = A.rpt[row], a1 = A.rpt[row + 1];
        if (a0 < 0 || a1 < a0 || a1 > A.nnz) {
            bad = true;
            a0 = a1 = 0;
        }
        long long f = 0;
        for (int j = a0 + lane; j < a1; j += 32) {
            const int b = A.col[j];
            if ((unsigned)b < (unsigned)K) {
                const int b0 = B.rpt[b], b1 = B.rpt[b + 1];
                if (b0 < 0 || b1 < b0)
                    bad = true;  // a negative length would wrap the unsigned total
                else
                    f += b1 - b0;
            } else {
                bad = true;
            }
        }
        f = brm::warp_sum(f);
        if (lane == 0) {
            // with valid CSR a row's count is at most nnz(B) <= INT_MAX; more
            // means repeated columns in the A row, reported, never clamped
            if (f > INT_MAX)
                big = true;
            else if (row_flop)
                row_flop[row] = (int)f;
            wsum += (unsigned long long)f;
        }
    }
    const unsigned long long ew = (__any_sync(brm::kFull, bad) ? kNaBadInput : 0ull) |
                                  (__any_sync(brm::kFull, big) ? kNaRowOverflow : 0ull);
    if (ew && lane == 0)
        atomicOr(&scratch[kNoAllocMaxBlocks + 1], ew);
    if (lane == 0)
        s_part[w] = wsum;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int i = 0; i < kNoAllocThreads / 32; i++)
            t += s_part[i];
        scratch[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kNoAllocThreads)
    k_flop_noalloc_total(int nblocks, unsigned long long *scratch)
{
    __shared__ unsigned long long s_part[kNoAllocThreads / 32];
    unsigned long long t = 0;
    for (int i = threadIdx.x; i < nblocks; i += kNoAllocThreads)
        t += scratch[i];
    t = brm::warp_sum(t);
    if ((threadIdx.x & 31) == 0)
        s_part[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int i = 0; i < kNoAllocThreads / 32; i++)
            s += s_part[i];
        scratch[kNoAllocMaxBlocks] = s;
    }
}

int scratch_for_current_device(unsigned long long **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return BRM_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices)
        return BRM_ERR_CAPACITY;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_dev[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            (void)cudaGetLastError();
            return BRM_ERR_CUDA;
        }
        g_noalloc_dev[dev] = (unsigned long long *)p;
    }
    *out = g_noalloc_dev[dev];
    return BRM_SUCCESS;
}

}  // namespace

extern "C" int brm_compute_flop_noalloc(const brm_csr *A, const brm_csr *B, int *row_flop,
                                        long long *products, void *stream)
{
    if (!A || !B || !products || !A->rpt || !B->rpt || A->M < 0 || B->M < 0 || A->nnz < 0 ||
        A->N != B->M || (A->nnz > 0 && !A->col))
        return BRM_ERR_INVALID_VALUE;
    if ((long long)A->M > kNoAllocMaxRows)
        return BRM_ERR_CAPACITY;  // the fixed scratch holds one partial per 64 rows
    *products = 0;
    if (A->M == 0)
        return BRM_SUCCESS;
    unsigned long long *scratch = nullptr;
    const int st = scratch_for_current_device(&scratch);
    if (st != BRM_SUCCESS)
        return st;
    cudaStream_t s = (cudaStream_t)stream;
    const int nblocks = (int)((A->M + kNoAllocRowsPerBlock - 1) / kNoAllocRowsPerBlock);
    cudaError_t e = cudaMemsetAsync(scratch + kNoAllocMaxBlocks + 1, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        k_flop_noalloc<<<nblocks, kNoAllocThreads, 0, s>>>(*A, *B, row_flop, scratch);
        k_flop_noalloc_total<<<1, kNoAllocThreads, 0, s>>>(nblocks, scratch);
        e = cudaGetLastError();
    }
    unsigned long long res[2] = {0, 0};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(res, scratch + kNoAllocMaxBlocks, sizeof(res), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return BRM_ERR_CUDA;
    }
    if (res[1] & kNaBadInput)
        return BRM_ERR_INVALID_CSR;
    if (res[1] & kNaRowOverflow)
        return BRM_ERR_OVERFLOW;
    *products = (long long)res[0];
    return BRM_SUCCESS;
}
