// brm_midwarp.cuh -- one warp per mid row: merged product keys, no block barriers.
//
// Rows with at most kMwF products (and at most kMidMaxK A entries, column
// range below 2^kMwRangeBits) are the bulk of regular products (a 27-point
// stencil squared: 729 products, 27 lists, 125 outputs per row) and of small
// uneven batches.  A warp takes a row at a time:
//
//   1. its nonempty lists (leaf order) into a warp-private table;
//   2. every product as a 32-bit key ((column - cmin) << 10 | product index)
//      in list-major order, i.e. leaf order (BRMerge-SpGEMM/inc/spgemm.h:
//      618-624: list l holds the l-th A entry's scaled B row);
//   3. a bottom-up merge of the sorted lists by key, ceil(log2 lists)
//      levels (merge path: every lane a contiguous share of the output), so
//      equal columns end in leaf order;
//   4. the runs of one column are listed and lane i reduces runs i, i + 32,
//      ... with the merge-tree rule (adjacent leaves join at their split
//      level: closed forms up to four leaves, a register shift-reduce beyond,
//      spgemm.h:639-707), values recomputed from A and B at this point.
//
// The same kernel counts the row (symbolic), writes it at crpt (Precise), at
// the row's product offset (Upper) or into the one-call scratch.
#pragma once

#include <climits>

#include "brm_common.cuh"
#include "brm_mid.cuh"
#include "brm_plan.h"

namespace brm {

enum MidWarpMode : int { kMwSymbolic = 0, kMwPrecise = 1, kMwUpper = 2, kMwScratch = 3 };

constexpr int kMwWarps = 12;
constexpr int kMwThreads = kMwWarps * 32;
constexpr int kMwIdxBits = 10;  // product index in the key (kMwF <= 1024)
static_assert(kMwF <= (1 << kMwIdxBits), "product index must fit the key");
static_assert(kMwRangeBits + kMwIdxBits <= 32, "keys are 32-bit");

struct MidWarpLayout {
    // keys, merged back and forth between k0 and k1; the free one then lists
    // the runs (up to kMwF + 1 entries)
    static constexpr size_t o_k0 = 0;
    static constexpr size_t o_k1 = o_k0 + mid_a16((kMwF + 1) * 4);
    static constexpr size_t o_plist = o_k1 + mid_a16((kMwF + 1) * 4);  // list of each product
    static constexpr size_t o_loff = o_plist + mid_a16(kMwF);           // list product offsets
    static constexpr size_t o_lbs = o_loff + mid_a16((kMidMaxK + 2) * 2);
    static constexpr size_t o_lleaf = o_lbs + (kMidMaxK + 1) * 4;
    static constexpr size_t per_warp = mid_a16(o_lleaf + kMidMaxK + 1);
    static constexpr size_t bytes = per_warp * kMwWarps;
};

// Merge-tree value of a run of n >= 1 products in leaf order (leaves below
// 2^(D-1)).
template <typename T, int D, typename GetLeaf, typename GetVal>
__device__ __forceinline__ T mw_run_value(int n, const GetLeaf &leaf, const GetVal &val)
{
    if (n == 1)
        return val(0);
    if (n == 2)
        return vadd(val(0), val(1));
    if (n == 3)
        return trie3(leaf(0), leaf(1), leaf(2), val(0), val(1), val(2));
    if (n == 4)
        return trie4(leaf(0), leaf(1), leaf(2), leaf(3), val(0), val(1), val(2), val(3));
    RegShiftReduce<T, D> sr;
    sr.init(leaf(0), val(0));
    for (int i = 1; i < n; i++)
        sr.push(leaf(i), val(i));
    return sr.finish();
}

// One level of the warp's bottom-up merge: runs of 2^L consecutive lists;
// runs 2m and 2m+1 merge into dst, a run without a right neighbour is
// copied.  The lane writes output positions [p0, p1).  Keys are unique
// (they hold the product index), so the merge is a plain merge of keys.
__device__ __forceinline__ void mw_merge_level(int L, const unsigned *__restrict__ src,
                                               unsigned *__restrict__ dst,
                                               const unsigned short *loff, int nl, int p0, int p1)
{
    if (p0 >= p1)
        return;
    int lo = 0, hi = nl - 1;  // list holding position p0
    while (lo < hi) {
        const int m = (lo + hi + 1) >> 1;
        if (loff[m] <= p0)
            lo = m;
        else
            hi = m - 1;
    }
    int j = lo;
    int p = p0;
    while (p < p1) {
        const int pg = (j >> L) & ~1;
        const int l0 = pg << L;
        const int l1 = min((pg + 1) << L, nl);
        const int l2 = min((pg + 2) << L, nl);
        const int ls = loff[l0], le = loff[l1], re = loff[l2];
        const int stop = min(p1, re);
        if (le == re) {
            for (; p < stop; p++)
                dst[p] = src[p];
        } else {
            const int na = le - ls, nb = re - le, d = p - ls;
            int a = max(0, d - nb), b = min(d, na);
            while (a < b) {
                const int m = (a + b) >> 1;
                if (src[ls + m] < src[le + d - 1 - m])
                    a = m + 1;
                else
                    b = m;
            }
            int ia = a, ib = d - a;
            unsigned ka = ia < na ? src[ls + ia] : 0xffffffffu;
            unsigned kb = ib < nb ? src[le + ib] : 0xffffffffu;
            for (; p < stop; p++) {
                if (ka < kb) {
                    dst[p] = ka;
                    ka = ++ia < na ? src[ls + ia] : 0xffffffffu;
                } else {
                    dst[p] = kb;
                    kb = ++ib < nb ? src[le + ib] : 0xffffffffu;
                }
            }
        }
        j = l2;
    }
}

template <typename T, int MODE>
__global__ void __launch_bounds__(kMwThreads) k_mid_warp(CsrDev A, CsrDev B, PlanDev P,
                                                         const int *crpt, int *ccol, T *cval)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char *ws = smem + (size_t)wid * MidWarpLayout::per_warp;
    unsigned *k0 = (unsigned *)(ws + MidWarpLayout::o_k0);
    unsigned *k1 = (unsigned *)(ws + MidWarpLayout::o_k1);
    unsigned char *plist = ws + MidWarpLayout::o_plist;
    unsigned short *loff = (unsigned short *)(ws + MidWarpLayout::o_loff);
    int *lbs = (int *)(ws + MidWarpLayout::o_lbs);
    unsigned char *lleaf = ws + MidWarpLayout::o_lleaf;
    const unsigned lt = lanemask_lt();
    const int M = A.M;
    const int n = P.cnt->bin_count[kBinMidWarp];
    const int *rows = P.rows + (size_t)kBinMidWarp * M;
    const int *__restrict__ bcol = B.col;
    const T *__restrict__ bval = (const T *)B.val;
    const T *__restrict__ aval = (const T *)A.val;
    const int gw = (blockIdx.x * kMwThreads + threadIdx.x) >> 5;
    const int nw = (gridDim.x * kMwThreads) >> 5;
    for (int it = gw; it < n; it += nw) {
        const int row = rows[it];
        if (row < P.r_lo || row >= P.r_hi)
            continue;
        const int a0 = A.rpt[row];
        const int k = A.rpt[row + 1] - a0;
        const int2 cr = P.crange[row];
        const int cmin = cr.x;
        // 1. nonempty lists in leaf order
        int nl = 0, F = 0;
        for (int jb = 0; jb < k; jb += 32) {
            const int j = jb + lane;
            const int len = j < k ? P.alen[a0 + j] : 0;
            const bool ne = len > 0;
            const unsigned nem = __ballot_sync(kFull, ne);
            const int inc = warp_incl_scan(len);
            const int tot = __shfl_sync(kFull, inc, 31);
            if (ne) {
                const int li = nl + __popc(nem & lt);
                loff[li] = (unsigned short)(F + inc - len);
                lbs[li] = P.abs[a0 + j];
                lleaf[li] = (unsigned char)j;
            }
            nl += __popc(nem);
            F += tot;
        }
        if (F > kMwF || cr.y - cmin >= (1 << kMwRangeBits)) {  // the analysis bins prevent this
            if (lane == 0)
                atomicOr(&P.cnt->err, kErrWindowOverflow);
            continue;
        }
        if (lane == 0)
            loff[nl] = (unsigned short)F;
        __syncwarp();
        // 2. keys in list-major (leaf) order: each list is sorted by key
        {
            int lo = 0, hi = nl - 1;  // list of product `lane`
            while (lo < hi) {
                const int m = (lo + hi + 1) >> 1;
                if (loff[m] <= lane)
                    lo = m;
                else
                    hi = m - 1;
            }
            int j = lo;
            for (int e = lane; e < F; e += 32) {
                while (e >= loff[j + 1])
                    j++;
                const int c = bcol[lbs[j] + (e - loff[j])];
                k0[e] = ((unsigned)(c - cmin) << kMwIdxBits) | (unsigned)e;
                plist[e] = (unsigned char)j;
            }
        }
        __syncwarp();
        // 3. bottom-up merge of the sorted lists (ceil(log2 nl) levels)
        unsigned *src = k0, *dst = k1;
        {
            const int per = (F + 31) >> 5;
            const int p0 = min(lane * per, F), p1 = min(p0 + per, F);
            const int levels = 32 - __clz(nl - 1);  // nl >= 2
            for (int L = 0; L < levels; L++) {
                mw_merge_level(L, src, dst, loff, nl, p0, p1);
                __syncwarp();
                unsigned *x = src;
                src = dst;
                dst = x;
            }
        }
        // 4. runs of one column: the heads (first product of each run) are
        //    listed in order, then lane i reduces runs i, i + 32, ... (its
        //    output goes to the row's position i: coalesced stores)
        int len = 0;
        for (int pb = 0; pb < F; pb += 32) {
            const int p = pb + lane;
            bool head = false;
            if (p < F)
                head = p == 0 || (src[p] >> kMwIdxBits) != (src[p - 1] >> kMwIdxBits);
            const unsigned hm = __ballot_sync(kFull, head);
            if (head)
                dst[len + __popc(hm & lt)] = (unsigned)p;
            len += __popc(hm);
        }
        if (lane == 0)
            dst[len] = (unsigned)F;
        __syncwarp();
        if (MODE == kMwSymbolic) {
            if (lane == 0)
                P.nnz[row] = len;
            continue;
        }
        long long base;
        if (MODE == kMwPrecise) {
            base = crpt[row];
            if (lane == 0 && len != crpt[row + 1] - crpt[row])
                atomicOr(&P.cnt->err, kErrNnzMismatch);
        } else if (MODE == kMwUpper) {
            base = P.scan_flop[row];
        } else {
            base = P.mid_pre[M] + P.mw_pre[row];
        }
        if ((MODE == kMwUpper || MODE == kMwScratch) && lane == 0)
            P.nnz[row] = len;
        const T *arow = aval + a0;
        constexpr unsigned imask = (1u << kMwIdxBits) - 1u;
        for (int h = lane; h < len; h += 32) {
            const int p = (int)dst[h], m = (int)dst[h + 1] - p;
            const unsigned *run = src + p;
            auto leaf = [&](int i) { return (int)lleaf[plist[run[i] & imask]]; };
            auto val = [&](int i) {
                const int e = (int)(run[i] & imask);
                const int j = plist[e];
                return vmul(arow[lleaf[j]], bval[lbs[j] + (e - loff[j])]);
            };
            // leaves below 32 need at most 5 stack entries below the top
            const T v = k <= 32 ? mw_run_value<T, 6>(m, leaf, val) : mw_run_value<T, 9>(m, leaf, val);
            ccol[base + h] = cmin + (int)(run[0] >> kMwIdxBits);
            cval[base + h] = v;
        }
        __syncwarp();
    }
}

template <typename T, int MODE>
inline void launch_mid_warp(const CsrDev &A, const CsrDev &B, const PlanDev &P, const int *crpt,
                            int *ccol, T *cval, int num_sms, cudaStream_t s)
{
    const size_t sm = MidWarpLayout::bytes;
    cudaFuncSetAttribute(k_mid_warp<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_mid_warp<T, MODE><<<num_sms * 2, kMwThreads, sm, s>>>(A, B, P, crpt, ccol, cval);
    count_launch();
}

}  // namespace brm
