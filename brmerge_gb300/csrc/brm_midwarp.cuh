// brm_midwarp.cuh -- one warp (or four) per mid row: merged product keys, no block barriers.
//
// Rows with at most kMg2F products (and at most kMidMaxK A entries, a column
// range below 2^kMwRangeBits / 2^kMgRangeBits) are the bulk of regular
// products (a 27-point stencil squared: 729 products, 27 lists, 125 outputs
// per row) and of uneven batches.  A warp (rows up to kMwF products) or a
// group of four warps takes a row at a time:
//
//   1. its nonempty lists (leaf order) into a warp-private table;
//   2. every product as a 32-bit key ((column - cmin) << 10 | product index)
//      in list-major order, i.e. leaf order (BRMerge-SpGEMM/inc/spgemm.h:
//      618-624: list l holds the l-th A entry's scaled B row);
//   3. the keys sorted: up to 128 products in registers by a bitonic
//      network across the warp, more by a bottom-up merge of the sorted
//      lists, ceil(log2 lists) levels (merge path: every lane a contiguous
//      share of the output); the keys are unique and equal columns end in
//      leaf order;
//   4. the runs of one column are listed and reduced with the merge-tree rule
//      (adjacent leaves join at their split level, a register shift-reduce,
//      spgemm.h:639-707), values recomputed from A and B at this point; the
//      products are split evenly over the lanes (a lane takes the runs that
//      start in its share), so long runs do not leave the other lanes idle.
//      Tile rows keep one lane per run (closed forms up to four leaves).
//
// The same kernel counts the row (symbolic), writes it at crpt (Precise), at
// the row's product offset (Upper) or into the one-call scratch.
#pragma once

#include <climits>

#include "brm_check.cuh"
#include "brm_common.cuh"
#include "brm_mid.cuh"
#include "brm_plan.h"

namespace brm {

enum MidWarpMode : int { kMwSymbolic = 0, kMwPrecise = 1, kMwUpper = 2, kMwScratch = 3 };

// Shapes (SID): a group of G warps works on one row at a time, GROUPS groups
// a CTA.  SID 1: one warp, rows of at most kMwF products; SID 4: four warps
// (named barriers) up to kMgF; SID 5: four warps up to kMg2F, two groups a
// CTA.  Keys are (column - cmin) << IDX | product index.
template <int SID>
struct MwShape;
template <>
struct MwShape<1> {
    static constexpr int W = 0;  // index of the shape's work counter
    static constexpr int G = 1;
    static constexpr int F = kMwF;
    static constexpr int IDX = 10;
    static constexpr int RANGE = kMwRangeBits;
    static constexpr int GROUPS = 12;
    static constexpr int BIN = kBinMidWarp;
    static constexpr int KMAX = kMwMaxK;
};
template <>
struct MwShape<4> {
    static constexpr int W = 1;
    static constexpr int G = 4;
    static constexpr int F = kMgF;
    static constexpr int IDX = 12;
    static constexpr int RANGE = kMgRangeBits;
    static constexpr int GROUPS = 3;
    static constexpr int BIN = kBinMidGroup;
    static constexpr int KMAX = kMwMaxK;
};
template <>
struct MwShape<5> {
    static constexpr int W = 2;
    static constexpr int G = 4;
    static constexpr int F = kMg2F;
    static constexpr int IDX = 13;
    static constexpr int RANGE = kMg2RangeBits;
    static constexpr int GROUPS = 2;
    static constexpr int BIN = kBinMidGroup2;
    static constexpr int KMAX = kMidMaxK;
};
constexpr int kMwThreads = 384;  // threads of the tile kernels
template <int SID>
constexpr int mw_threads()
{
    return MwShape<SID>::GROUPS * MwShape<SID>::G * 32;
}
static_assert(MwShape<1>::F <= (1 << MwShape<1>::IDX) && MwShape<1>::RANGE + MwShape<1>::IDX <= 32,
              "warp keys are 32-bit");
static_assert(MwShape<4>::F <= (1 << MwShape<4>::IDX) && MwShape<4>::RANGE + MwShape<4>::IDX <= 32,
              "group keys are 32-bit");
static_assert(MwShape<5>::F <= (1 << MwShape<5>::IDX) && MwShape<5>::RANGE + MwShape<5>::IDX <= 32,
              "group keys are 32-bit");

template <int SID>
struct MidWarpLayout {
    static constexpr int G = MwShape<SID>::G;
    static constexpr int FM = MwShape<SID>::F;
    // keys, merged back and forth between k0 and k1; the free one then lists
    // the runs (up to FM + 1 entries)
    static constexpr size_t o_k0 = 0;
    static constexpr size_t o_k1 = o_k0 + mid_a16((FM + 1) * 4);
    static constexpr size_t o_plist = o_k1 + mid_a16((FM + 1) * 4);  // list of each product
    static constexpr size_t o_loff = o_plist + mid_a16(FM);           // list product offsets
    static constexpr int KM = MwShape<SID>::KMAX;
    static constexpr size_t o_lbs = o_loff + mid_a16((KM + 2) * 2);
    static constexpr size_t o_lleaf = o_lbs + (KM + 1) * 4;
    static constexpr size_t o_gs = o_lleaf + mid_a16(KM + 1);  // group scan scratch, next row
    static constexpr size_t per_group = mid_a16(o_gs + 4 * (G + 1));
    static constexpr size_t bytes = per_group * MwShape<SID>::GROUPS;
};

template <int G>
__device__ __forceinline__ void grp_sync(int gid)
{
    if (G == 1)
        __syncwarp();
    else
        asm volatile("bar.sync %0, %1;" ::"r"(gid + 1), "r"(G * 32) : "memory");
}

// Exclusive scan of one int per thread of the group; *total gets the sum.
template <int G>
__device__ __forceinline__ int grp_excl_scan(int v, int *gs, int gid, int *total)
{
    const int lane = threadIdx.x & 31;
    const int inc = warp_incl_scan(v);
    if (G == 1) {
        *total = __shfl_sync(kFull, inc, 31);
        return inc - v;
    }
    const int w = (threadIdx.x >> 5) % G;
    grp_sync<G>(gid);  // gs may still be read by a previous scan
    if (lane == 31)
        gs[w] = inc;
    grp_sync<G>(gid);
    int off = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < G; i++) {
        const int x = gs[i];
        off += i < w ? x : 0;
        tot += x;
    }
    *total = tot;
    return off + inc - v;
}

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

// One level of the group's bottom-up merge: runs of 2^L consecutive lists;
// runs 2m and 2m+1 merge into dst, a run without a right neighbour is
// copied.  The thread writes output positions [p0, p1).  Keys are unique
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
            int ia = ls + a, ib = le + d - a;  // next positions in src
            unsigned ka = ia < le ? src[ia] : 0xffffffffu;
            unsigned kb = ib < re ? src[ib] : 0xffffffffu;
            for (; p < stop; p++) {
                // branch-free step: one load, lanes stay converged
                const bool ta = ka < kb;
                dst[p] = ta ? ka : kb;
                const int nx = ta ? ++ia : ++ib;
                const unsigned kn = nx < (ta ? le : re) ? src[nx] : 0xffffffffu;
                ka = ta ? kn : ka;
                kb = ta ? kb : kn;
            }
        }
        j = l2;
    }
}

// Sorts the warp's 32 * KPL keys in registers (bitonic network; key i =
// lane * KPL + q), ascending.
template <int KPL>
__device__ __forceinline__ void warp_bitonic_keys(unsigned (&key)[KPL])
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 2; k <= 32 * KPL; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= KPL) {
                const int lj = j / KPL;
#pragma unroll
                for (int q = 0; q < KPL; q++) {
                    const unsigned o = __shfl_xor_sync(kFull, key[q], lj);
                    const int i = lane * KPL + q;
                    const bool up = (i & k) == 0, lower = (i & j) == 0;
                    key[q] = (lower == up) ? min(key[q], o) : max(key[q], o);
                }
            } else {
#pragma unroll
                for (int q = 0; q < KPL; q++) {
                    if (q & j)
                        continue;
                    const int i = lane * KPL + q;
                    const bool up = (i & k) == 0;
                    const unsigned a = key[q], b = key[q | j];
                    key[q] = up ? min(a, b) : max(a, b);
                    key[q | j] = up ? max(a, b) : min(a, b);
                }
            }
        }
    }
}

// Sorts keys[0, F) (F <= 32 * KPL) of a warp in place through registers.
template <int KPL>
__device__ __forceinline__ void warp_sort_small(unsigned *keys, int F)
{
    const int lane = threadIdx.x & 31;
    unsigned key[KPL];
#pragma unroll
    for (int q = 0; q < KPL; q++) {
        const int i = lane * KPL + q;
        key[q] = i < F ? keys[i] : 0xffffffffu;
    }
    __syncwarp();
    warp_bitonic_keys<KPL>(key);
#pragma unroll
    for (int q = 0; q < KPL; q++) {
        const int i = lane * KPL + q;
        if (i < F)
            keys[i] = key[q];
    }
    __syncwarp();
}

// Values of all runs with the products split evenly over the NT threads:
// thread t takes the runs that start among products [t F / NT, (t + 1) F / NT)
// and walks their products in order (run h covers key[head[h], head[h + 1]),
// head[len] = F), gathering GB products ahead of the merge-tree reduction.
// Every thread then handles about F / NT products however long the runs are
// (a lane per run leaves most lanes idle while one reduces a long run).
template <typename T, int NT, int IDX, int D, int GB>
__device__ __forceinline__ void mw_reduce_balanced(const unsigned *key, const unsigned *head,
                                                   int len, int F, int t,
                                                   const unsigned char *plist,
                                                   const unsigned char *lleaf, const int *lbs,
                                                   const unsigned short *loff,
                                                   const T *__restrict__ arow,
                                                   const T *__restrict__ bval, int cmin, int *ccol,
                                                   T *cval, Counters *cnt, long long bnnz)
{
    constexpr unsigned imask = (1u << IDX) - 1u;
    // first run that starts at or after product q (len if none)
    auto first_run = [&](int q) {
        int lo = 0, hi = len;
        while (lo < hi) {
            const int m = (lo + hi) >> 1;
            if ((int)head[m] < q)
                lo = m + 1;
            else
                hi = m;
        }
        return lo;
    };
    const int h0 = first_run((int)((long long)t * F / NT));
    const int h1 = first_run((int)((long long)(t + 1) * F / NT));
    if (h0 >= h1)
        return;
    const int pend = (int)head[h1];
    int h = h0;
    int next = (int)head[h0 + 1];
    RegShiftReduce<T, D> sr;
    for (int p0 = (int)head[h0]; p0 < pend; p0 += GB) {
        int lf[GB];
        T v[GB];
#pragma unroll
        for (int q = 0; q < GB; q++) {
            lf[q] = 0;
            v[q] = T(0);
            if (p0 + q < pend) {
                const int e = (int)(key[p0 + q] & imask);
                const int j = plist[e];
                lf[q] = lleaf[j];
                const long long bi = (long long)lbs[j] + (e - loff[j]);
                v[q] = BRM_IN(cnt, bi, bnnz) ? vmul(arow[lf[q]], bval[bi]) : T(0);
            }
        }
#pragma unroll
        for (int q = 0; q < GB; q++) {
            const int p = p0 + q;
            if (p < pend) {
                if (p == (int)head[h0]) {
                    sr.init(lf[q], v[q]);
                } else if (p == next) {  // run h is complete
                    ccol[h] = cmin + (int)(key[head[h]] >> IDX);
                    cval[h] = sr.finish();
                    h++;
                    next = (int)head[h + 1];
                    sr.init(lf[q], v[q]);
                } else {
                    sr.push(lf[q], v[q]);
                }
            }
        }
    }
    ccol[h] = cmin + (int)(key[head[h]] >> IDX);
    cval[h] = sr.finish();
}

template <typename T, int MODE, int SID>
__global__ void __launch_bounds__(mw_threads<SID>(), 2) k_mid_warp(CsrDev A, CsrDev B, PlanDev P,
                                                               const int *crpt, int *ccol, T *cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    using S = MwShape<SID>;
    using L = MidWarpLayout<SID>;
    constexpr int G = S::G;
    constexpr int NT = 32 * G;
    constexpr int IDX = S::IDX;
    extern __shared__ __align__(16) unsigned char smem[];
    const int gid = threadIdx.x / NT, t = threadIdx.x % NT;
    unsigned char *ws = smem + (size_t)gid * L::per_group;
    unsigned *k0 = (unsigned *)(ws + L::o_k0);
    unsigned *k1 = (unsigned *)(ws + L::o_k1);
    unsigned char *plist = ws + L::o_plist;
    unsigned short *loff = (unsigned short *)(ws + L::o_loff);
    int *lbs = (int *)(ws + L::o_lbs);
    unsigned char *lleaf = ws + L::o_lleaf;
    int *gs = (int *)(ws + L::o_gs);
    const int M = A.M;
    const int n = P.cnt->bin_count[S::BIN];
    const int *rows = P.rows + (size_t)S::BIN * M;
    const int *__restrict__ bcol = B.col;
    const T *__restrict__ bval = (const T *)B.val;
    const T *__restrict__ aval = (const T *)A.val;
    // rows are taken one at a time from a counter (the classes span a
    // fourfold range of products, so a fixed share per group leaves a long
    // tail); gs[G] passes the item to the group
    int *work = &P.cnt->work_mw[S::W];
    for (;;) {
        if (t == 0)
            gs[G] = atomicAdd(work, 1);
        grp_sync<G>(gid);
        const int it = gs[G];
        grp_sync<G>(gid);  // every thread has the item before gs[G] is reused
        if (it >= n)
            break;
        const int row = rows[it];
        if (row < P.r_lo || row >= P.r_hi)
            continue;
        const int a0 = A.rpt[row];
        const int k = A.rpt[row + 1] - a0;
        const int2 cr = P.crange[row];
        const int cmin = cr.x;
        // 1. nonempty lists in leaf order (count << 16 | products, scanned)
        int nl = 0, F = 0;
        for (int jb = 0; jb < k; jb += NT) {
            const int j = jb + t;
            const int len = j < k ? P.alen[a0 + j] : 0;
            const int x = len > 0 ? (1 << 16) + len : 0;
            int tot;
            const int ex = grp_excl_scan<G>(x, gs, gid, &tot);
            if (len > 0) {
                const int li = nl + (ex >> 16);
                loff[li] = (unsigned short)(F + (ex & 0xffff));
                lbs[li] = P.abs[a0 + j];
                lleaf[li] = (unsigned char)j;
            }
            nl += tot >> 16;
            F += tot & 0xffff;
        }
        // the analysis bins prevent this
        if (F > S::F || k > S::KMAX || cr.y - cmin >= (1 << S::RANGE)) {
            if (t == 0)
                atomicOr(&P.cnt->err, kErrWindowOverflow);
            grp_sync<G>(gid);
            continue;
        }
        if (t == 0)
            loff[nl] = (unsigned short)F;
        grp_sync<G>(gid);
        // 2. keys in list-major (leaf) order: each list is sorted by key
        {
            int lo = 0, hi = nl - 1;  // list of product t
            while (lo < hi) {
                const int m = (lo + hi + 1) >> 1;
                if (loff[m] <= t)
                    lo = m;
                else
                    hi = m - 1;
            }
            int j = lo;
            constexpr int KU = 4;  // column loads in flight per thread
            for (int eb = t; eb < F; eb += KU * NT) {
                int c[KU], jj[KU];
#pragma unroll
                for (int u = 0; u < KU; u++) {
                    const int e = eb + u * NT;
                    c[u] = 0;
                    if (e < F) {
                        while (e >= loff[j + 1])
                            j++;
                        const long long bi = (long long)lbs[j] + (e - loff[j]);
                        c[u] = BRM_IN(P.cnt, bi, B.nnz) ? bcol[bi] : cmin;
                    }
                    jj[u] = j;
                }
#pragma unroll
                for (int u = 0; u < KU; u++) {
                    const int e = eb + u * NT;
                    if (e < F) {
                        k0[e] = ((unsigned)(c[u] - cmin) << IDX) | (unsigned)e;
                        plist[e] = (unsigned char)jj[u];
                    }
                }
            }
        }
        grp_sync<G>(gid);
        // 3. sort by key: small rows of one warp in registers (bitonic),
        //    others by a bottom-up merge of the sorted lists (ceil(log2 nl)
        //    levels, nl >= 2)
        unsigned *src = k0, *dst = k1;
        const int per = (F + NT - 1) / NT;
        const int p0 = min(t * per, F), p1 = min(p0 + per, F);
        if (G == 1 && F <= 64) {
            warp_sort_small<2>(src, F);
        } else if (G == 1 && F <= 128) {
            warp_sort_small<4>(src, F);
        } else {
            const int levels = 32 - __clz(nl - 1);
            for (int lv = 0; lv < levels; lv++) {
                mw_merge_level(lv, src, dst, loff, nl, p0, p1);
                grp_sync<G>(gid);
                unsigned *x = src;
                src = dst;
                dst = x;
            }
        }
        // 4. runs of one column: each thread finds the heads (first products
        //    of runs) in its share, they are listed in order, and every
        //    thread reduces the runs that start in its share of the products
        int nh = 0;
        for (int p = p0; p < p1; p++)
            nh += p == 0 || (src[p] >> IDX) != (src[p - 1] >> IDX);
        int len;
        int hx = grp_excl_scan<G>(nh, gs, gid, &len);
        for (int p = p0; p < p1; p++)
            if (p == 0 || (src[p] >> IDX) != (src[p - 1] >> IDX))
                dst[hx++] = (unsigned)p;
        if (t == 0)
            dst[len] = (unsigned)F;
        grp_sync<G>(gid);
        if (MODE == kMwSymbolic) {
            if (t == 0)
                P.nnz[row] = len;
            grp_sync<G>(gid);
            continue;
        }
        long long base;
        if (MODE == kMwPrecise) {
            base = crpt[row];
            if (t == 0 && len != crpt[row + 1] - crpt[row])
                atomicOr(&P.cnt->err, kErrNnzMismatch);
        } else if (MODE == kMwUpper) {
            base = P.scan_flop[row];
        } else {
            base = P.mid_pre[M] + P.mw_pre[row];
        }
        if ((MODE == kMwUpper || MODE == kMwScratch) && t == 0)
            P.nnz[row] = len;
        // the row's output must lie inside C (or the scratch): checked build
        if (!BRM_IN(P.cnt, base + len - 1, MODE == kMwScratch ? P.mid_cap : P.c_cap)) {
            grp_sync<G>(gid);
            continue;
        }
        // gathers in flight: two runs a thread within 80 registers, four
        // with 128
        if (k <= 32)
            mw_reduce_balanced<T, NT, IDX, 6, 4>(src, dst, len, F, t, plist, lleaf, lbs, loff,
                                                 aval + a0, bval, cmin, ccol + base, cval + base,
                                                 P.cnt, B.nnz);
        else
            mw_reduce_balanced<T, NT, IDX, (S::KMAX <= 64 ? 7 : 9), 4>(
                src, dst, len, F, t, plist, lleaf, lbs, loff, aval + a0, bval, cmin, ccol + base,
                cval + base, P.cnt, B.nnz);
        grp_sync<G>(gid);
    }
    // the last group of the launch clears the counters for the next launch
    // (its own taken items and every other group's are ordered before)
    if (t == 0) {
        __threadfence();
        if (atomicAdd(&P.cnt->done_mw[S::W], 1) == (int)gridDim.x * S::GROUPS - 1) {
            atomicExch(work, 0);
            atomicExch(&P.cnt->done_mw[S::W], 0);
        }
    }
}

// ---------------------------------------------------------------------------
// Tile rows: at most kMtF products, half a warp (16 lanes) each, four keys a
// lane sorted by a bitonic network that stays inside the half warp, so a
// warp works on two rows at once.
// ---------------------------------------------------------------------------
constexpr int kMtTW = 16;  // lanes per row

// Shape of a tile class: KPL keys a lane, FM = 16 * KPL products at most.
template <int KPL>
struct MtShape;
template <>
struct MtShape<4> {
    static constexpr int FM = kMtF;
    static constexpr int IDX = 6;
    static constexpr int BIN = kBinMidTile;
};
template <>
struct MtShape<8> {
    static constexpr int FM = kMt2F;
    static constexpr int IDX = 7;
    static constexpr int BIN = kBinMidTile2;
};
static_assert(kMtF == kMtTW * 4 && kMt2F == kMtTW * 8, "tile shapes");
static_assert(kMtRangeBits + 7 <= 32, "tile keys are 32-bit");

template <int FM>
struct MidTileLayout {
    static constexpr size_t o_key = 0;                            // sorted keys
    static constexpr size_t o_head = o_key + FM * 4;               // run starts, + 1
    static constexpr size_t o_lbs = o_head + (FM + 1) * 4;         // list B starts
    static constexpr size_t o_loff = o_lbs + FM * 4;               // list product offsets
    static constexpr size_t o_plist = o_loff + mid_a16((FM + 1) * 2);
    static constexpr size_t o_lleaf = o_plist + FM;
    static constexpr size_t per_tile = mid_a16(o_lleaf + FM);
};

template <typename T, int MODE, int KPL>
__global__ void __launch_bounds__(kMwThreads, 2) k_mid_tile(CsrDev A, CsrDev B, PlanDev P,
                                                         const int *crpt, int *ccol, T *cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    using S = MtShape<KPL>;
    using TL = MidTileLayout<S::FM>;
    constexpr int TW = kMtTW, IDX = S::IDX, kMtF = S::FM;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int lt = lane & (TW - 1);
    const int tb = lane & ~(TW - 1);                      // tile's first lane
    const unsigned gm = ((1u << TW) - 1u) << tb;          // tile's lanes
    const unsigned ltm = (1u << lt) - 1u;                 // tile lanes below this one
    const int tile = threadIdx.x / TW;
    unsigned char *ws = smem + (size_t)tile * TL::per_tile;
    unsigned *skey = (unsigned *)(ws + TL::o_key);
    unsigned *shead = (unsigned *)(ws + TL::o_head);
    int *lbs = (int *)(ws + TL::o_lbs);
    unsigned short *loff = (unsigned short *)(ws + TL::o_loff);
    unsigned char *plist = ws + TL::o_plist;
    unsigned char *lleaf = ws + TL::o_lleaf;
    const int M = A.M;
    const int n = P.cnt->bin_count[S::BIN];
    const int *rows = P.rows + (size_t)S::BIN * M;
    const int *__restrict__ bcol = B.col;
    const T *__restrict__ bval = (const T *)B.val;
    const T *__restrict__ aval = (const T *)A.val;
    const int t0 = blockIdx.x * (kMwThreads / TW) + tile;
    const int nt = gridDim.x * (kMwThreads / TW);
    // both tiles of a warp run the same number of iterations, so the sort
    // network (full-warp shuffles) always has every lane
    for (int itb = t0 - (tile & 1); itb < n; itb += nt) {
        const int it = itb + (tile & 1);
        const bool live = it < n;
        const int row = live ? rows[it] : 0;
        const bool act = live && row >= P.r_lo && row < P.r_hi;
        int a0 = 0, k = 0, cmin = 0;
        if (act) {
            a0 = A.rpt[row];
            k = A.rpt[row + 1] - a0;
            cmin = P.crange[row].x;
        }
        // 1. nonempty lists in leaf order
        int nl = 0, F = 0;
        for (int jb = 0; jb < k; jb += TW) {
            const int j = jb + lt;
            const int len = j < k ? P.alen[a0 + j] : 0;
            const unsigned nem = (__ballot_sync(gm, len > 0) >> tb) & ((1u << TW) - 1u);
            int inc = len;
#pragma unroll
            for (int o = 1; o < TW; o <<= 1) {
                const int x = __shfl_up_sync(gm, inc, o, TW);
                if (lt >= o)
                    inc += x;
            }
            const int tot = __shfl_sync(gm, inc, TW - 1, TW);
            if (len > 0 && F + inc <= kMtF) {
                const int li = nl + __popc(nem & ltm);
                loff[li] = (unsigned short)(F + inc - len);
                lbs[li] = P.abs[a0 + j];
                lleaf[li] = (unsigned char)j;
            }
            nl += __popc(nem);
            F += tot;
        }
        const bool ok = act && F <= kMtF && nl >= 1;
        if (act && !ok && lt == 0)
            atomicOr(&P.cnt->err, kErrWindowOverflow);  // the analysis bins prevent this
        if (lt == 0 && ok)
            loff[nl] = (unsigned short)F;
        __syncwarp(gm);
        // 2. keys into registers: key q of lane lt is product lt * KPL + q
        unsigned key[KPL];
#pragma unroll
        for (int q = 0; q < KPL; q++) {
            const int i = lt * KPL + q;
            key[q] = 0xffffffffu;
            if (ok && i < F) {
                int lo = 0, hi = nl - 1;
                while (lo < hi) {
                    const int m = (lo + hi + 1) >> 1;
                    if (loff[m] <= i)
                        lo = m;
                    else
                        hi = m - 1;
                }
                const long long bi = (long long)lbs[lo] + (i - loff[lo]);
                const int c = BRM_IN(P.cnt, bi, B.nnz) ? bcol[bi] : cmin;
                key[q] = ((unsigned)(c - cmin) << IDX) | (unsigned)i;
                plist[i] = (unsigned char)lo;
            }
        }
        // 3. bitonic sort of the tile's TW * KPL keys (partners stay in the tile)
#pragma unroll
        for (int kk = 2; kk <= TW * KPL; kk <<= 1) {
#pragma unroll
            for (int j = kk >> 1; j > 0; j >>= 1) {
                if (j >= KPL) {
                    const int lj = j / KPL;
#pragma unroll
                    for (int q = 0; q < KPL; q++) {
                        const unsigned o = __shfl_xor_sync(kFull, key[q], lj);
                        const int i = lt * KPL + q;
                        const bool up = (i & kk) == 0, lower = (i & j) == 0;
                        key[q] = (lower == up) ? min(key[q], o) : max(key[q], o);
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < KPL; q++) {
                        if (q & j)
                            continue;
                        const int i = lt * KPL + q;
                        const bool up = (i & kk) == 0;
                        const unsigned a = key[q], b = key[q | j];
                        key[q] = up ? min(a, b) : max(a, b);
                        key[q | j] = up ? max(a, b) : min(a, b);
                    }
                }
            }
        }
        if (!ok)
            continue;
#pragma unroll
        for (int q = 0; q < KPL; q++) {
            const int i = lt * KPL + q;
            if (i < F)
                skey[i] = key[q];
        }
        __syncwarp(gm);
        // 4. runs of one column (heads listed in order), lane i reduces runs
        //    i, i + TW, ...
        int nh = 0;
#pragma unroll
        for (int q = 0; q < KPL; q++) {
            const int p = lt * KPL + q;
            if (p < F)
                nh += p == 0 || (skey[p] >> IDX) != (skey[p - 1] >> IDX);
        }
        int hx = nh;
#pragma unroll
        for (int o = 1; o < TW; o <<= 1) {
            const int x = __shfl_up_sync(gm, hx, o, TW);
            if (lt >= o)
                hx += x;
        }
        const int len = __shfl_sync(gm, hx, TW - 1, TW);
        hx -= nh;
#pragma unroll
        for (int q = 0; q < KPL; q++) {
            const int p = lt * KPL + q;
            if (p < F && (p == 0 || (skey[p] >> IDX) != (skey[p - 1] >> IDX)))
                shead[hx++] = (unsigned)p;
        }
        if (lt == 0)
            shead[len] = (unsigned)F;
        __syncwarp(gm);
        if (MODE == kMwSymbolic) {
            if (lt == 0)
                P.nnz[row] = len;
            __syncwarp(gm);
            continue;
        }
        long long base;
        if (MODE == kMwPrecise) {
            base = crpt[row];
            if (lt == 0 && len != crpt[row + 1] - crpt[row])
                atomicOr(&P.cnt->err, kErrNnzMismatch);
        } else if (MODE == kMwUpper) {
            base = P.scan_flop[row];
        } else {
            base = P.mid_pre[M] + P.mw_pre[row];
        }
        if ((MODE == kMwUpper || MODE == kMwScratch) && lt == 0)
            P.nnz[row] = len;
        const T *arow = aval + a0;
        constexpr unsigned imask = (1u << IDX) - 1u;
        // the row's output must lie inside C (or the scratch): checked build
        const bool out_in = BRM_IN(P.cnt, base + len - 1, MODE == kMwScratch ? P.mid_cap : P.c_cap);
        for (int h = out_in ? lt : len; h < len; h += TW) {
            const int p = (int)shead[h], m = (int)shead[h + 1] - p;
            const unsigned *run = skey + p;
            auto leaf = [&](int i) { return (int)lleaf[plist[run[i] & imask]]; };
            auto val = [&](int i) {
                const int e = (int)(run[i] & imask);
                const int j = plist[e];
                const long long bi = (long long)lbs[j] + (e - loff[j]);
                return BRM_IN(P.cnt, bi, B.nnz) ? vmul(arow[lleaf[j]], bval[bi]) : T(0);
            };
            const T v = k <= 32 ? mw_run_value<T, 6>(m, leaf, val) : mw_run_value<T, 9>(m, leaf, val);
            ccol[base + h] = cmin + (int)(run[0] >> IDX);
            cval[base + h] = v;
        }
        __syncwarp(gm);
    }
}

template <typename T, int MODE, int SID>
inline void launch_mid_group(const CsrDev &A, const CsrDev &B, const PlanDev &P, const int *crpt,
                             int *ccol, T *cval, int num_sms, cudaStream_t s)
{
    const size_t sm = MidWarpLayout<SID>::bytes;
    cudaFuncSetAttribute(k_mid_warp<T, MODE, SID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_mid_warp<T, MODE, SID><<<num_sms * 2, mw_threads<SID>(), sm, s>>>(A, B, P, crpt, ccol,
                                                                         cval);
    count_launch();
}

template <typename T, int MODE, int KPL>
inline void launch_mid_tile(const CsrDev &A, const CsrDev &B, const PlanDev &P, const int *crpt,
                            int *ccol, T *cval, int num_sms, cudaStream_t s)
{
    const size_t sm = (size_t)(kMwThreads / kMtTW) * MidTileLayout<MtShape<KPL>::FM>::per_tile;
    cudaFuncSetAttribute(k_mid_tile<T, MODE, KPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_mid_tile<T, MODE, KPL><<<num_sms * 4, kMwThreads, sm, s>>>(A, B, P, crpt, ccol, cval);
    count_launch();
}

// The warp rows, the four-warp group rows and the tile rows of one mode.
// which: kMidGroups (the four-warp groups), kMidWarps (warp and tile rows) or
// both; classes without rows are not launched.
template <typename T, int MODE>
inline void launch_mid_warp(const CsrDev &A, const CsrDev &B, const PlanDev &P, const int *crpt,
                            int *ccol, T *cval, int num_sms, cudaStream_t s,
                            int which = kMidGroups | kMidWarps)
{
    if (which & kMidGroups) {
        if (plan_live(P, live_bit(kBinMidGroup2)))
            launch_mid_group<T, MODE, 5>(A, B, P, crpt, ccol, cval, num_sms, s);
        if (plan_live(P, live_bit(kBinMidGroup)))
            launch_mid_group<T, MODE, 4>(A, B, P, crpt, ccol, cval, num_sms, s);
    }
    if (which & kMidWarps) {
        if (plan_live(P, live_bit(kBinMidWarp)))
            launch_mid_group<T, MODE, 1>(A, B, P, crpt, ccol, cval, num_sms, s);
        if (plan_live(P, live_bit(kBinMidTile2)))
            launch_mid_tile<T, MODE, 8>(A, B, P, crpt, ccol, cval, num_sms, s);
        if (plan_live(P, live_bit(kBinMidTile)))
            launch_mid_tile<T, MODE, 4>(A, B, P, crpt, ccol, cval, num_sms, s);
    }
}

}  // namespace brm
