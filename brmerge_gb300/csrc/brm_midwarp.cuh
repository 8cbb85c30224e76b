// brm_midwarp.cuh -- one warp per mid row: radix-ordered products, no block barriers.
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
//   3. a stable LSD radix sort of the keys on the column bits (at most 9
//      bits a pass; a warp ranks equal digits in lane order from one ballot
//      per digit bit, so equal columns keep leaf order);
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

constexpr int kMwWarps = 8;
constexpr int kMwThreads = kMwWarps * 32;
constexpr int kMwIdxBits = 10;  // product index in the key (kMwF <= 1024)
constexpr int kMwDigit = 9;     // radix digit width at most
constexpr int kMwBins = 1 << kMwDigit;
static_assert(kMwF <= (1 << kMwIdxBits), "product index must fit the key");
static_assert(kMwRangeBits + kMwIdxBits <= 32, "keys are 32-bit");

struct MidWarpLayout {
    // keys (sorted in place between k0 and k1; the free one then lists the
    // runs, up to kMwF + 1 entries)
    static constexpr size_t o_k0 = 0;
    static constexpr size_t o_k1 = o_k0 + mid_a16((kMwF + 1) * 4);
    static constexpr size_t o_addr = o_k1 + mid_a16((kMwF + 1) * 4);   // B position per product
    static constexpr size_t o_leaf = o_addr + kMwF * 4;                // leaf per product
    static constexpr size_t o_hist = o_leaf + mid_a16(kMwF);           // digit counts
    static constexpr size_t o_loff = o_hist + kMwBins * 4;             // list product offsets
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

template <typename T, int MODE>
__global__ void __launch_bounds__(kMwThreads) k_mid_warp(CsrDev A, CsrDev B, PlanDev P,
                                                         const int *crpt, int *ccol, T *cval)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char *ws = smem + (size_t)wid * MidWarpLayout::per_warp;
    unsigned *k0 = (unsigned *)(ws + MidWarpLayout::o_k0);
    unsigned *k1 = (unsigned *)(ws + MidWarpLayout::o_k1);
    int *paddr = (int *)(ws + MidWarpLayout::o_addr);
    unsigned char *pleaf = ws + MidWarpLayout::o_leaf;
    int *hist = (int *)(ws + MidWarpLayout::o_hist);
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
        // 2. keys in list-major (leaf) order
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
                const int addr = lbs[j] + (e - loff[j]);
                const int c = bcol[addr];
                k0[e] = ((unsigned)(c - cmin) << kMwIdxBits) | (unsigned)e;
                paddr[e] = addr;
                pleaf[e] = lleaf[j];
            }
        }
        __syncwarp();
        // 3. stable radix sort on the column bits
        const int rb = cr.y > cmin ? 32 - __clz(cr.y - cmin) : 0;
        unsigned *src = k0, *dst = k1;
        if (rb > 0) {
            const int passes = (rb + kMwDigit - 1) / kMwDigit;
            const int width = (rb + passes - 1) / passes;
            const unsigned dmask = (1u << width) - 1u;
            const int nbins = 1 << width;
            for (int ps = 0; ps < passes; ps++) {
                const int shift = kMwIdxBits + ps * width;
                for (int b = lane; b < nbins; b += 32)
                    hist[b] = 0;
                __syncwarp();
                for (int e = lane; e < F; e += 32)
                    atomicAdd(&hist[(src[e] >> shift) & dmask], 1);
                __syncwarp();
                {
                    // exclusive scan of the counts: lane owns bins [lane*per, +per)
                    const int per = nbins >> 5 > 0 ? nbins >> 5 : 1;
                    int s = 0;
                    for (int q = 0; q < per; q++) {
                        const int b = lane * per + q;
                        if (b < nbins)
                            s += hist[b];
                    }
                    int run = warp_incl_scan(s) - s;
                    for (int q = 0; q < per; q++) {
                        const int b = lane * per + q;
                        if (b < nbins) {
                            const int c = hist[b];
                            hist[b] = run;
                            run += c;
                        }
                    }
                }
                __syncwarp();
                for (int eb = 0; eb < F; eb += 32) {
                    const int e = eb + lane;
                    const bool ok = e < F;
                    const unsigned key = ok ? src[e] : 0u;
                    const int d = ok ? (int)((key >> shift) & dmask) : 0;
                    // lanes with the same digit: one ballot per digit bit
                    // (several times the throughput of __match_any_sync here)
                    unsigned peers = __ballot_sync(kFull, ok);
                    for (int b = 0; b < width; b++) {
                        const bool bit = (d >> b) & 1;
                        const unsigned m = __ballot_sync(kFull, bit);
                        peers &= bit ? m : ~m;
                    }
                    int pos = 0;
                    if (ok)
                        pos = hist[d] + __popc(peers & lt);
                    __syncwarp();
                    if (ok && (peers >> lane) == 1u)  // last lane of its digit group
                        hist[d] += __popc(peers);
                    __syncwarp();
                    if (ok)
                        dst[pos] = key;
                }
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
            auto leaf = [&](int i) { return (int)pleaf[run[i] & imask]; };
            auto val = [&](int i) {
                const int e = (int)(run[i] & imask);
                return vmul(arow[pleaf[e]], bval[paddr[e]]);
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
