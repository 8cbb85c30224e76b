// brm_hash.cu -- hash SpGEMM comparator (no merge-order values).
//
// The competitor the BRMerge paper measures against: Nagasaka et al.'s
// binned hash SpGEMM (Existing-SpGEMM/inc/hash_mult.h:1028-1057,
// HashSpGEMM<sortOutput = true>, bins of BIN.h:77-186): per row, a symbolic
// pass counts the distinct columns with a hash table keyed by column
// ((key * 107) & (size - 1), linear probing, hash_mult.h:96-118), and a
// numeric pass accumulates the products per column and stores the row sorted
// by column.  The structure of C is identical to BRMerge's; the values are
// sums in an order the hardware picks (shared/global atomics), so they agree
// with the merge-tree values only to rounding.  It measures what the
// merge-tree order costs.
//
// GB300 form, by products F of a row:
//   F <= 32           one warp per row, products in registers: sort by
//                     column (shuffle network), reduce equal columns
//   F <= kHashWarpF   one warp per row, warp-private shared-memory table
//   F <= kHashCtaF    one CTA per row, shared-memory table
//   larger            one CTA per row with a dense accumulator (value array
//                     and column bitmap over the row's column range, from a
//                     per-CTA pool): the bitmap scan emits columns in order
// Outputs of the table bins are sorted with a bitonic network in shared
// memory.
#include <algorithm>
#include <climits>
#include <cstring>

#include "brm_common.cuh"
#include "brm_kernels.h"
#include "brmerge.h"

namespace brm {
namespace {

constexpr int kHashScale = 107;   // hash_mult.h:22
constexpr int kHashWarpF = 512;   // products of the warp-table bin
constexpr int kHashWarpT = 1024;  // its table slots (>= 2 F)
constexpr int kHashCtaF = 4096;   // products of the CTA-table bin
constexpr int kHashCtaT = 8192;   // its table slots
constexpr int kHashThreads = 256;
constexpr int kHashWarps = kHashThreads / 32;

enum HashBin : int { kHB0 = 0, kHB32 = 1, kHBWarp = 2, kHBCta = 3, kHBDense = 4, kHBins = 5 };

struct HashCnt {
    int bin_count[kHBins];
    int work[kHBins];  // dynamic row counters
    int err;
    int pad;
};

struct HashPlan {
    int M;
    int *flop;       // [M]
    int *nnz;        // [M]
    int *rows;       // [kHBins * M]
    int2 *crange;    // [M] column range of dense rows
    HashCnt *cnt;
    unsigned long long *dense_pool;  // bitmap words of the dense accumulators
    void *dense_val;                 // values of the dense accumulators
    int dense_cols;                  // columns of one accumulator (N)
    int dense_slots;                 // accumulators in the pool
};

__device__ __forceinline__ int hash_slot(int key, int mask) { return (key * kHashScale) & mask; }

__device__ __forceinline__ int next_pow2(int x)
{
    int p = 1;
    while (p < x)
        p <<= 1;
    return p;
}

// Products per row and bins (warp per row).
__global__ void k_hash_rows(CsrDev A, CsrDev B, HashPlan P)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int row = gw; row < A.M; row += nw) {
        const int a0 = A.rpt[row], a1 = A.rpt[row + 1];
        long long f = 0;
        int cmin = INT_MAX, cmax = -1;
        for (int j = a0 + lane; j < a1; j += 32) {
            const int k = A.col[j];
            if ((unsigned)k >= (unsigned)B.M) {
                atomicOr(&P.cnt->err, 2);  // the host stops before any other kernel
                continue;
            }
            const int b0 = B.rpt[k], b1 = B.rpt[k + 1];
            if (b1 < b0) {
                atomicOr(&P.cnt->err, 2);
                continue;
            }
            f += b1 - b0;
            if (b1 > b0) {
                const int c0 = B.col[b0], c1 = B.col[b1 - 1];
                if (c0 < 0 || c1 >= B.N)
                    atomicOr(&P.cnt->err, 2);
                cmin = min(cmin, c0);
                cmax = max(cmax, c1);
            }
        }
        f = warp_sum(f);
        cmin = warp_min(cmin);
        cmax = warp_max(cmax);
        if (lane == 0) {
            if (f > INT_MAX) {
                atomicOr(&P.cnt->err, 1);
                f = INT_MAX;
            }
            const int F = (int)f;
            P.flop[row] = F;
            const int b = F == 0 ? kHB0 : F <= 32 ? kHB32 : F <= kHashWarpF ? kHBWarp
                          : F <= kHashCtaF ? kHBCta : kHBDense;
            if (b == kHB0)
                P.nnz[row] = 0;
            const int pos = atomicAdd(&P.cnt->bin_count[b], 1);
            P.rows[(long long)b * P.M + pos] = row;
            P.crange[row] = make_int2(cmin, cmax);
        }
    }
}

// ---- rows of at most 32 products: one warp, registers ------------------------

// Bitonic sort of one (key, value) per lane across the warp, ascending keys.
template <typename T>
__device__ __forceinline__ void warp_sort_kv(int &key, T &val)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int ok = __shfl_xor_sync(kFull, key, j);
            const T ov = __shfl_xor_sync(kFull, val, j);
            const bool up = (lane & k) == 0;
            const bool lower = (lane & j) == 0;
            const bool take = lower == up ? ok < key : ok > key;
            if (take) {
                key = ok;
                val = ov;
            }
        }
    }
}

template <typename T, bool NUMERIC>
__global__ void k_hash_warp32(CsrDev A, CsrDev B, HashPlan P, const int *crpt, int *ccol, T *cval)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int n = P.cnt->bin_count[kHB32];
    const int *rows = P.rows + (long long)kHB32 * P.M;
    const T *aval = (const T *)A.val;
    const T *bval = (const T *)B.val;
    for (int it = gw; it < n; it += nw) {
        const int row = rows[it];
        // product `lane` of the row (lists in A order)
        int key = INT_MAX;
        T v = T(0);
        {
            int p = lane;
            for (int j = A.rpt[row]; j < A.rpt[row + 1]; j++) {
                const int k = A.col[j];
                const int b0 = B.rpt[k], len = B.rpt[k + 1] - b0;
                if (p >= 0 && p < len) {
                    key = B.col[b0 + p];
                    if (NUMERIC)
                        v = vmul(aval[j], bval[b0 + p]);
                }
                p -= len;
            }
        }
        warp_sort_kv(key, v);
        const int prev = __shfl_up_sync(kFull, key, 1);
        const bool head = key != INT_MAX && (lane == 0 || prev != key);
        const unsigned heads = __ballot_sync(kFull, head);
        if (!NUMERIC) {
            if (lane == 0)
                P.nnz[row] = __popc(heads);
            continue;
        }
        // each run of equal keys is contiguous: its head adds the run in lane
        // order (every lane takes part in every shuffle)
        T acc = v;
        const unsigned after = heads & ~((2u << lane) - 1u);  // heads after this lane
        const int end = after ? __ffs(after) - 1 : 32;
        for (int q = 1; q < 32; q++) {
            const T t = __shfl_sync(kFull, v, q);
            const int kq = __shfl_sync(kFull, key, q);
            if (head && q > lane && q < end && kq == key)
                acc = vadd(acc, t);
        }
        if (head) {
            const int r = __popc(heads & ((1u << lane) - 1u));
            const long long o = (long long)crpt[row] + r;
            ccol[o] = key;
            cval[o] = acc;
        }
    }
}

// ---- table bins ------------------------------------------------------------

// Bitonic sort of n (<= P, P a power of two) key/value pairs in shared
// memory by `nt` threads starting at thread t0 (sync = warp or block).
template <typename T, bool BLOCK>
__device__ __forceinline__ void smem_sort_kv(int *k, T *v, int P, int t, int nt)
{
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = t; i < (P >> 1); i += nt) {
                const int lo = 2 * i - (i & (stride - 1));
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const int a = k[lo], b = k[hi];
                if ((a > b) == up) {
                    k[lo] = b;
                    k[hi] = a;
                    const T x = v[lo];
                    v[lo] = v[hi];
                    v[hi] = x;
                }
            }
            if (BLOCK)
                __syncthreads();
            else
                __syncwarp();
        }
    }
}

template <typename T>
struct WarpTableLayout {
    static constexpr size_t keys = (size_t)kHashWarps * kHashWarpT * 4;
    static constexpr size_t vals = (size_t)kHashWarps * kHashWarpT * sizeof(T);
    static constexpr size_t bytes = keys + vals;
};

// One warp per row, warp-private table of kHashWarpT slots.
template <typename T, bool NUMERIC>
__global__ void __launch_bounds__(kHashThreads)
    k_hash_warptab(CsrDev A, CsrDev B, HashPlan P, const int *crpt, int *ccol, T *cval)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int *keys = (int *)smem + wid * kHashWarpT;
    T *vals = (T *)(smem + WarpTableLayout<T>::keys) + wid * kHashWarpT;
    const int n = P.cnt->bin_count[kHBWarp];
    const int *rows = P.rows + (long long)kHBWarp * P.M;
    const T *aval = (const T *)A.val;
    const T *bval = (const T *)B.val;
    for (;;) {
        int it = 0;
        if (lane == 0)
            it = atomicAdd(&P.cnt->work[kHBWarp], 1);
        it = __shfl_sync(kFull, it, 0);
        if (it >= n)
            break;
        const int row = rows[it];
        const int F = P.flop[row];
        const int Tn = min(next_pow2(2 * F), kHashWarpT);
        const int mask = Tn - 1;
        for (int s = lane; s < Tn; s += 32) {
            keys[s] = -1;
            if (NUMERIC)
                vals[s] = T(0);
        }
        __syncwarp();
        int cnt = 0;
        for (int j = A.rpt[row]; j < A.rpt[row + 1]; j++) {
            const int k = A.col[j];
            const int b0 = B.rpt[k], b1 = B.rpt[k + 1];
            const T a = NUMERIC ? aval[j] : T(0);
            for (int q = b0 + lane; q < b1; q += 32) {
                const int key = B.col[q];
                int h = hash_slot(key, mask);
                for (;;) {
                    const int old = atomicCAS(&keys[h], -1, key);
                    if (old == -1 || old == key) {
                        if (NUMERIC)
                            atomicAdd(&vals[h], vmul(a, bval[q]));
                        else
                            cnt += old == -1;
                        break;
                    }
                    h = (h + 1) & mask;
                }
            }
        }
        __syncwarp();
        if (!NUMERIC) {
            cnt = warp_sum(cnt);
            if (lane == 0)
                P.nnz[row] = cnt;
            continue;
        }
        // compact to the front (any order), pad, sort by column
        const int nz = P.nnz[row];
        const int Ps = next_pow2(max(nz, 1));
        int base = 0;
        for (int s0 = 0; s0 < Tn; s0 += 32) {
            const int s = s0 + lane;
            const int key = s < Tn ? keys[s] : -1;
            const T v = s < Tn ? vals[s] : T(0);
            const unsigned occ = __ballot_sync(kFull, key != -1);
            __syncwarp();
            if (key != -1) {
                const int d = base + __popc(occ & lanemask_lt());
                keys[d] = key;  // d <= s: never overwrites an unread slot
                vals[d] = v;
            }
            base += __popc(occ);
            __syncwarp();
        }
        for (int s = nz + lane; s < Ps; s += 32)
            keys[s] = INT_MAX;
        __syncwarp();
        smem_sort_kv<T, false>(keys, vals, Ps, lane, 32);
        const long long o = crpt[row];
        for (int s = lane; s < nz; s += 32) {
            ccol[o + s] = keys[s];
            cval[o + s] = vals[s];
        }
        __syncwarp();
    }
}

template <typename T>
struct CtaTableLayout {
    static constexpr size_t keys = (size_t)kHashCtaT * 4;
    static constexpr size_t bytes = keys + (size_t)kHashCtaT * sizeof(T) + 64;
};

// One CTA per row, table of kHashCtaT slots.
template <typename T, bool NUMERIC>
__global__ void __launch_bounds__(kHashThreads)
    k_hash_ctatab(CsrDev A, CsrDev B, HashPlan P, const int *crpt, int *ccol, T *cval)
{
    extern __shared__ __align__(16) unsigned char smem[];
    int *keys = (int *)smem;
    T *vals = (T *)(smem + CtaTableLayout<T>::keys);
    int *misc = (int *)(smem + CtaTableLayout<T>::bytes - 64);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int n = P.cnt->bin_count[kHBCta];
    const int *rows = P.rows + (long long)kHBCta * P.M;
    const T *aval = (const T *)A.val;
    const T *bval = (const T *)B.val;
    for (;;) {
        if (tid == 0)
            misc[0] = atomicAdd(&P.cnt->work[kHBCta], 1);
        __syncthreads();
        const int it = misc[0];
        if (it >= n)
            break;
        const int row = rows[it];
        const int F = P.flop[row];
        const int Tn = min(next_pow2(2 * F), kHashCtaT);
        const int mask = Tn - 1;
        for (int s = tid; s < Tn; s += kHashThreads) {
            keys[s] = -1;
            if (NUMERIC)
                vals[s] = T(0);
        }
        if (tid == 0)
            misc[1] = 0;
        __syncthreads();
        int cnt = 0;
        // warps take the lists of the row in turn
        for (int j = A.rpt[row] + wid; j < A.rpt[row + 1]; j += kHashWarps) {
            const int k = A.col[j];
            const int b0 = B.rpt[k], b1 = B.rpt[k + 1];
            const T a = NUMERIC ? aval[j] : T(0);
            for (int q = b0 + lane; q < b1; q += 32) {
                const int key = B.col[q];
                int h = hash_slot(key, mask);
                for (;;) {
                    const int old = atomicCAS(&keys[h], -1, key);
                    if (old == -1 || old == key) {
                        if (NUMERIC)
                            atomicAdd(&vals[h], vmul(a, bval[q]));
                        else
                            cnt += old == -1;
                        break;
                    }
                    h = (h + 1) & mask;
                }
            }
        }
        if (!NUMERIC) {
            cnt = warp_sum(cnt);
            if (lane == 0 && cnt)
                atomicAdd(&misc[1], cnt);
            __syncthreads();
            if (tid == 0)
                P.nnz[row] = misc[1];
            __syncthreads();
            continue;
        }
        __syncthreads();
        // compact into the upper half of the table (slots Tn/2..) is not
        // free in general, so compact in place in two steps: gather the
        // occupied slots' (key, value) into registers chunk by chunk
        const int nz = P.nnz[row];
        const int Ps = next_pow2(max(nz, 1));
        for (int s0 = 0; s0 < Tn; s0 += kHashThreads) {
            const int s = s0 + tid;
            const int key = s < Tn ? keys[s] : -1;
            const T v = s < Tn ? vals[s] : T(0);
            const unsigned occ = __ballot_sync(kFull, key != -1);
            if (lane == 0)
                misc[8 + wid] = __popc(occ);
            __syncthreads();
            int wbase = misc[1];
            for (int w = 0; w < wid; w++)
                wbase += misc[8 + w];
            int tot = misc[1];
            for (int w = 0; w < kHashWarps; w++)
                tot += misc[8 + w];
            __syncthreads();
            if (key != -1) {
                const int d = wbase + __popc(occ & lanemask_lt());
                keys[d] = key;  // d <= s
                vals[d] = v;
            }
            if (tid == 0)
                misc[1] = tot;
            __syncthreads();
        }
        for (int s = nz + tid; s < Ps; s += kHashThreads)
            keys[s] = INT_MAX;
        __syncthreads();
        smem_sort_kv<T, true>(keys, vals, Ps, tid, kHashThreads);
        const long long o = crpt[row];
        for (int s = tid; s < nz; s += kHashThreads) {
            ccol[o + s] = keys[s];
            cval[o + s] = vals[s];
        }
        __syncthreads();
    }
}

// ---- dense accumulator for the heaviest rows ---------------------------------

template <typename T, bool NUMERIC>
__global__ void __launch_bounds__(kHashThreads)
    k_hash_dense(CsrDev A, CsrDev B, HashPlan P, const int *crpt, int *ccol, T *cval)
{
    __shared__ int misc[2];
    __shared__ long long ws[kHashWarps + 1];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int n = P.cnt->bin_count[kHBDense];
    const int *rows = P.rows + (long long)kHBDense * P.M;
    const T *aval = (const T *)A.val;
    const T *bval = (const T *)B.val;
    const long long words = ((long long)P.dense_cols + 63) >> 6;
    unsigned long long *bm = P.dense_pool + (long long)blockIdx.x * words;
    T *acc = (T *)P.dense_val + (long long)blockIdx.x * P.dense_cols;
    for (;;) {
        if (tid == 0)
            misc[0] = atomicAdd(&P.cnt->work[kHBDense], 1);
        __syncthreads();
        const int it = misc[0];
        __syncthreads();
        if (it >= n)
            break;
        const int row = rows[it];
        const int2 cr = P.crange[row];
        // (bitmap and accumulator are clear between rows)
        for (int j = A.rpt[row] + wid; j < A.rpt[row + 1]; j += kHashWarps) {
            const int k = A.col[j];
            const int b0 = B.rpt[k], b1 = B.rpt[k + 1];
            const T a = NUMERIC ? aval[j] : T(0);
            for (int q = b0 + lane; q < b1; q += 32) {
                const int c = B.col[q];
                if ((unsigned)c > (unsigned)cr.y || c < cr.x) {
                    atomicOr(&P.cnt->err, 2);  // B row not sorted or out of range
                    continue;
                }
                atomicOr(&bm[c >> 6], 1ull << (c & 63));
                if (NUMERIC)
                    atomicAdd(&acc[c], vmul(a, bval[q]));
            }
        }
        __syncthreads();
        // scan the bitmap over the row's range: columns in order
        const long long w0 = cr.x >> 6, w1 = (cr.y >> 6) + 1;
        long long base = NUMERIC ? (long long)crpt[row] : 0;
        for (long long wb = w0; wb < w1; wb += kHashThreads) {
            const long long w = wb + tid;
            const unsigned long long bits = w < w1 ? bm[w] : 0ull;
            long long tot;
            const long long ex = block_excl_scan<kHashThreads, long long>(__popcll(bits), ws, &tot);
            if (NUMERIC) {
                unsigned long long b = bits;
                long long o = base + ex;
                while (b) {
                    const int t = __ffsll((long long)b) - 1;
                    b &= b - 1;
                    const int c = (int)(w * 64 + t);
                    ccol[o] = c;
                    cval[o] = acc[c];
                    acc[c] = T(0);
                    o++;
                }
            }
            if (w < w1 && bits)
                bm[w] = 0ull;
            base += tot;
        }
        if (!NUMERIC && tid == 0)
            P.nnz[row] = (int)base;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------
int cuda_st(cudaError_t e)
{
    if (e == cudaSuccess)
        return BRM_SUCCESS;
    (void)cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? BRM_ERR_ALLOC : BRM_ERR_CUDA;
}

template <typename T, bool NUMERIC>
void launch_phase(const CsrDev &A, const CsrDev &B, const HashPlan &P, const int *hbins,
                  const int *crpt, int *ccol, void *cval, int num_sms, cudaStream_t s)
{
    T *cv = (T *)cval;
    if (hbins[kHB32]) {
        const int g = std::min((hbins[kHB32] + 7) / 8, num_sms * 16);
        k_hash_warp32<T, NUMERIC><<<g, 256, 0, s>>>(A, B, P, crpt, ccol, cv);
        count_launch();
    }
    if (hbins[kHBWarp]) {
        const size_t sm = WarpTableLayout<T>::bytes;
        cudaFuncSetAttribute(k_hash_warptab<T, NUMERIC>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        const int g = std::min((hbins[kHBWarp] + kHashWarps - 1) / kHashWarps, num_sms * 2);
        k_hash_warptab<T, NUMERIC><<<g, kHashThreads, sm, s>>>(A, B, P, crpt, ccol, cv);
        count_launch();
    }
    if (hbins[kHBCta]) {
        const size_t sm = CtaTableLayout<T>::bytes;
        cudaFuncSetAttribute(k_hash_ctatab<T, NUMERIC>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        const int g = std::min(hbins[kHBCta], num_sms * 2);
        k_hash_ctatab<T, NUMERIC><<<g, kHashThreads, sm, s>>>(A, B, P, crpt, ccol, cv);
        count_launch();
    }
    if (hbins[kHBDense]) {
        const int g = std::min(hbins[kHBDense], P.dense_slots);
        k_hash_dense<T, NUMERIC><<<g, kHashThreads, 0, s>>>(A, B, P, crpt, ccol, cv);
        count_launch();
    }
}

}  // namespace
}  // namespace brm

extern "C" int brm_hash_device(brm_context ctx, brm_dtype dtype, const brm_csr *A,
                               const brm_csr *B, int **crpt_, int **ccol_, void **cval_,
                               int *cnnz_)
{
    using namespace brm;
    if (!ctx || !A || !B || !crpt_ || !ccol_ || !cval_ || !cnnz_)
        return BRM_ERR_INVALID_VALUE;
    if (dtype != BRM_F64 && dtype != BRM_F32)
        return BRM_ERR_INVALID_VALUE;
    if (A->M < 0 || A->N < 0 || B->M < 0 || B->N < 0 || A->N != B->M)
        return BRM_ERR_INVALID_VALUE;
    cudaStream_t s = context_stream(ctx);
    const int num_sms = context_num_sms(ctx);
    const int M = A->M;
    CsrDev a{A->M, A->N, A->nnz, A->rpt, A->col, A->val};
    CsrDev b{B->M, B->N, B->nnz, B->rpt, B->col, B->val};
    const size_t vb = dtype == BRM_F64 ? 8 : 4;
    // workspace: flop, nnz, rows, crange, counters, scan scratch (each
    // piece starts on a 256-byte boundary)
    const size_t mm = (size_t)std::max(M, 1);
    const size_t piece[6] = {mm * 4, mm * 4, mm * 4 * kHBins, mm * 8, sizeof(HashCnt),
                             scan_tmp_bytes(M)};
    size_t ws_bytes = 0;
    for (size_t p : piece)
        ws_bytes += (p + 255) & ~size_t(255);
    char *ws = nullptr;
    int st = cuda_st(cudaMallocAsync((void **)&ws, ws_bytes, s));
    if (st != BRM_SUCCESS)
        return st;
    HashPlan P{};
    P.M = M;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = ws + off;
        off += (bytes + 255) & ~size_t(255);
        return (void *)p;
    };
    P.flop = (int *)take(piece[0]);
    P.nnz = (int *)take(piece[1]);
    P.rows = (int *)take(piece[2]);
    P.crange = (int2 *)take(piece[3]);
    P.cnt = (HashCnt *)take(piece[4]);
    void *stmp = take(piece[5]);
    int *crpt = nullptr, *ccol = nullptr;
    void *cval = nullptr;
    unsigned long long *pool = nullptr;
    void *pool_val = nullptr;
    HashCnt hc{};
    auto fail = [&](int code) {
        if (crpt)
            cudaFreeAsync(crpt, s);
        if (ccol)
            cudaFreeAsync(ccol, s);
        if (cval)
            cudaFreeAsync(cval, s);
        if (pool)
            cudaFreeAsync(pool, s);
        if (pool_val)
            cudaFreeAsync(pool_val, s);
        cudaFreeAsync(ws, s);
        return code;
    };
    st = cuda_st(cudaMemsetAsync(P.cnt, 0, sizeof(HashCnt), s));
    if (st == BRM_SUCCESS)
        st = cuda_st(cudaMallocAsync((void **)&crpt, 4 * (mm + 1), s));
    if (st != BRM_SUCCESS)
        return fail(st);
    if (M > 0) {
        k_hash_rows<<<num_sms * 8, 256, 0, s>>>(a, b, P);
        count_launch();
    }
    st = cuda_st(cudaMemcpyAsync(&hc, P.cnt, sizeof(hc), cudaMemcpyDeviceToHost, s));
    if (st == BRM_SUCCESS)
        st = cuda_st(cudaStreamSynchronize(s));
    if (st != BRM_SUCCESS)
        return fail(st);
    if (hc.err)
        return fail((hc.err & 2) ? BRM_ERR_INVALID_CSR : BRM_ERR_OVERFLOW);
    // dense accumulators: one per CTA of the dense bin, within a memory budget
    if (hc.bin_count[kHBDense]) {
        const long long words = ((long long)B->N + 63) >> 6;
        const long long per = words * 8 + (long long)B->N * (long long)vb;
        const long long budget = 4ll << 30;
        const int slots = (int)std::max(1ll, std::min<long long>(num_sms * 2, budget / std::max(per, 1ll)));
        P.dense_cols = B->N;
        P.dense_slots = std::min(slots, hc.bin_count[kHBDense]);
        st = cuda_st(cudaMallocAsync((void **)&pool, (size_t)words * 8 * P.dense_slots, s));
        if (st == BRM_SUCCESS)
            st = cuda_st(cudaMallocAsync(&pool_val, (size_t)B->N * vb * P.dense_slots, s));
        if (st == BRM_SUCCESS)
            st = cuda_st(cudaMemsetAsync(pool, 0, (size_t)words * 8 * P.dense_slots, s));
        if (st == BRM_SUCCESS)
            st = cuda_st(cudaMemsetAsync(pool_val, 0, (size_t)B->N * vb * P.dense_slots, s));
        if (st != BRM_SUCCESS)
            return fail(st);
        P.dense_pool = pool;
        P.dense_val = pool_val;
    }
    // symbolic
    if (dtype == BRM_F64)
        launch_phase<double, false>(a, b, P, hc.bin_count, nullptr, nullptr, nullptr, num_sms, s);
    else
        launch_phase<float, false>(a, b, P, hc.bin_count, nullptr, nullptr, nullptr, num_sms, s);
    Counters *c2 = nullptr;
    st = cuda_st(cudaMallocAsync((void **)&c2, sizeof(Counters), s));
    if (st != BRM_SUCCESS)
        return fail(st);
    cudaMemsetAsync(c2, 0, sizeof(Counters), s);
    launch_scan_i32(P.nnz, crpt, M, c2, stmp, s);
    Counters h2{};
    st = cuda_st(cudaMemcpyAsync(&h2, c2, sizeof(h2), cudaMemcpyDeviceToHost, s));
    cudaFreeAsync(c2, s);
    if (st == BRM_SUCCESS)
        st = cuda_st(cudaStreamSynchronize(s));
    if (st != BRM_SUCCESS)
        return fail(st);
    if ((h2.err & kErrOverflow) || h2.cnnz > INT_MAX)
        return fail(BRM_ERR_OVERFLOW);
    const int cnnz = (int)h2.cnnz;
    st = cuda_st(cudaMallocAsync((void **)&ccol, 4 * (size_t)std::max(cnnz, 1), s));
    if (st == BRM_SUCCESS)
        st = cuda_st(cudaMallocAsync(&cval, vb * (size_t)std::max(cnnz, 1), s));
    if (st == BRM_SUCCESS)
        st = cuda_st(cudaMemsetAsync(P.cnt->work, 0, sizeof(hc.work), s));
    if (st != BRM_SUCCESS)
        return fail(st);
    // numeric
    if (dtype == BRM_F64)
        launch_phase<double, true>(a, b, P, hc.bin_count, crpt, ccol, cval, num_sms, s);
    else
        launch_phase<float, true>(a, b, P, hc.bin_count, crpt, ccol, cval, num_sms, s);
    st = cuda_st(cudaMemcpyAsync(&hc, P.cnt, sizeof(hc), cudaMemcpyDeviceToHost, s));
    if (st == BRM_SUCCESS)
        st = cuda_st(cudaStreamSynchronize(s));
    if (st != BRM_SUCCESS)
        return fail(st);
    if (hc.err)
        return fail(BRM_ERR_INVALID_CSR);
    if (pool)
        cudaFreeAsync(pool, s);
    if (pool_val)
        cudaFreeAsync(pool_val, s);
    cudaFreeAsync(ws, s);
    *crpt_ = crpt;
    *ccol_ = ccol;
    *cval_ = cval;
    *cnnz_ = cnnz;
    return BRM_SUCCESS;
}
