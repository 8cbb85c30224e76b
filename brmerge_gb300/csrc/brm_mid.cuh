// brm_mid.cuh -- batched kernels for mid rows (kWarpMaxFlop < products, small weight).
//
// Most rows of a power-law product have a few nonempty lists and almost no
// repeated columns, and there are tens of thousands of them; one CTA per row
// would spend its time in barriers.  These kernels pack consecutive mid rows
// into batches (at most kMidCap products and kMidMaxLists nonempty lists) and
// process a whole batch per CTA pass:
//
//   * symbolic: every product's column goes into a per-row open-addressing
//     hash table in shared memory; the number of successful inserts is the
//     row's exact nnz (the reference counts the same way, with a linear-probing
//     table, BRMerge-SpGEMM/inc/spgemm.h:528-556);
//   * numeric: the products of every row are staged in list-major order (list
//     l = leaf l of the row's merge tree) and sorted by column with a stable
//     bottom-up merge of the already sorted lists (merge path, ceil(log2 n)
//     levels for n nonempty lists); runs of equal columns then hold their
//     contributions in increasing leaf order and one thread per output column
//     evaluates the merge tree with ShiftReduce (spgemm.h:639-707).  Because a
//     batch holds consecutive rows, its output is written in one ordered sweep.
//
// Product gathers are issued in groups of kGatherBatch independent loads per
// thread before any of them is used, so each thread keeps several L2 requests
// in flight instead of waiting on one at a time.
#pragma once

#include <climits>

#include "brm_check.cuh"
#include "brm_common.cuh"
#include "brm_plan.h"
#include "brm_rows.cuh"

namespace brm {

constexpr int kGatherBatch = 8;

// Shared tables of one batch: its rows ("slots") and their nonempty lists.
struct MidBatch {
    int *s_row;   // [kMidMaxRows] row of each slot
    int *s_a0;    // [kMidMaxRows] arpt[row]
    int *s_kb;    // [kMidMaxRows+1] prefix of A-row lengths
    int *s_lb;    // [kMidMaxRows+1] first list of each slot
    int *loff;    // [kMidMaxLists+1] product offset of each nonempty list
    int *lbs;     // [kMidMaxLists] start of the list's B row
    unsigned char *lslot;  // [kMidMaxLists]
    unsigned char *lleaf;  // [kMidMaxLists] leaf (A-row position) of each list
    int *misc;    // [8] scalars: 0 nslots, 1 nlists, 2 nprod, 4 batch index
};

constexpr size_t mid_a16(size_t x) { return (x + 15) & ~size_t(15); }

template <typename T>
struct MidNumLayout {
    static constexpr size_t o_col = 0;
    static constexpr size_t o_val = o_col + mid_a16(kMidCap * 4);
    static constexpr size_t o_idx0 = o_val + mid_a16(kMidCap * sizeof(T));
    static constexpr size_t o_idx1 = o_idx0 + mid_a16(kMidCap * 2);
    static constexpr size_t o_lidx = o_idx1 + mid_a16(kMidCap * 2);
    static constexpr size_t o_loff = o_lidx + mid_a16(kMidCap * 2);
    static constexpr size_t o_lbs = o_loff + mid_a16((kMidMaxLists + 1) * 4);
    static constexpr size_t o_lslot = o_lbs + mid_a16(kMidMaxLists * 4);
    static constexpr size_t o_lleaf = o_lslot + mid_a16(kMidMaxLists);
    static constexpr size_t o_srow = o_lleaf + mid_a16(kMidMaxLists);
    static constexpr size_t o_sa0 = o_srow + mid_a16(kMidMaxRows * 4);
    static constexpr size_t o_skb = o_sa0 + mid_a16(kMidMaxRows * 4);
    static constexpr size_t o_slb = o_skb + mid_a16((kMidMaxRows + 1) * 4);
    static constexpr size_t o_shb = o_slb + mid_a16((kMidMaxRows + 1) * 4);
    static constexpr size_t o_head = o_shb + mid_a16((kMidMaxRows + 1) * 4);
    static constexpr size_t o_ws = o_head + mid_a16(kMidCap / 8);
    static constexpr size_t o_misc = o_ws + mid_a16((kMidThreads / 32 + 1) * 8);
    static constexpr size_t bytes = o_misc + 64;
};

constexpr int kMidHashCap = 4 * kMidCap;  // hash slots per batch (load factor <= 2/3 per row)

struct MidSymLayout {
    static constexpr size_t o_tab = 0;
    static constexpr size_t o_loff = o_tab + mid_a16(kMidHashCap * 4);
    static constexpr size_t o_lbs = o_loff + mid_a16((kMidMaxLists + 1) * 4);
    static constexpr size_t o_lslot = o_lbs + mid_a16(kMidMaxLists * 4);
    static constexpr size_t o_lleaf = o_lslot + mid_a16(kMidMaxLists);
    static constexpr size_t o_srow = o_lleaf + mid_a16(kMidMaxLists);
    static constexpr size_t o_sa0 = o_srow + mid_a16(kMidMaxRows * 4);
    static constexpr size_t o_skb = o_sa0 + mid_a16(kMidMaxRows * 4);
    static constexpr size_t o_slb = o_skb + mid_a16((kMidMaxRows + 1) * 4);
    static constexpr size_t o_hbase = o_slb + mid_a16((kMidMaxRows + 1) * 4);
    static constexpr size_t o_cnt = o_hbase + mid_a16((kMidMaxRows + 1) * 4);
    static constexpr size_t o_ws = o_cnt + mid_a16(kMidMaxRows * 4);
    static constexpr size_t o_misc = o_ws + mid_a16((kMidThreads / 32 + 1) * 8);
    static constexpr size_t bytes = o_misc + 64;
};

// Number of tree levels that merge n sorted runs pairwise into one.
__device__ __forceinline__ int ceil_log2(int n) { return n <= 1 ? 0 : 32 - __clz(n - 1); }

// Index of the last entry <= key in the non-decreasing arr[0..n) (arr[0] <= key).
__device__ __forceinline__ int last_le(const int *arr, int n, int key)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (arr[mid] <= key)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <typename T, typename L>
__device__ __forceinline__ MidBatch mid_tables(unsigned char *smem)
{
    MidBatch t;
    t.s_row = (int *)(smem + L::o_srow);
    t.s_a0 = (int *)(smem + L::o_sa0);
    t.s_kb = (int *)(smem + L::o_skb);
    t.s_lb = (int *)(smem + L::o_slb);
    t.loff = (int *)(smem + L::o_loff);
    t.lbs = (int *)(smem + L::o_lbs);
    t.lslot = (unsigned char *)(smem + L::o_lslot);
    t.lleaf = (unsigned char *)(smem + L::o_lleaf);
    t.misc = (int *)(smem + L::o_misc);
    return t;
}

// Loads the batch's rows and nonempty lists into the shared tables.
// Returns false (uniformly) if the batch does not fit the tables.
__device__ __forceinline__ bool mid_setup(const CsrDev &A, const PlanDev &P, int r0, int r1,
                                          MidBatch &t, long long *ws)
{
    constexpr int NT = kMidThreads;
    const int tid = threadIdx.x;
    // slots: the mid rows of [r0, r1), in row order
    int carry = 0;
    for (int rb = r0; rb < r1; rb += NT) {
        const int r = rb + tid;
        const int f = r < r1 ? P.mid_flop[r] : 0;
        long long tot;
        const int ex = (int)block_excl_scan<NT, long long>(f > 0 ? 1 : 0, ws, &tot) + carry;
        if (f > 0 && ex < kMidMaxRows)
            t.s_row[ex] = r;
        carry += (int)tot;
    }
    const int nslots = carry;
    if (nslots > kMidMaxRows) {
        if (tid == 0)
            atomicOr(&P.cnt->err, kErrWindowOverflow);
        return false;
    }
    __syncthreads();
    int k = 0;
    if (tid < nslots) {
        const int r = t.s_row[tid];
        const int a0 = A.rpt[r];
        t.s_a0[tid] = a0;
        k = A.rpt[r + 1] - a0;
    }
    long long ktot;
    const int kb = (int)block_excl_scan<NT, long long>(k, ws, &ktot);
    if (tid < nslots)
        t.s_kb[tid] = kb;
    if (tid == 0)
        t.s_kb[nslots] = (int)ktot;
    __syncthreads();
    // nonempty lists of all slots, slot-major then leaf order
    int lcarry = 0, pcarry = 0;
    for (int ib = 0; ib < (int)ktot; ib += NT) {
        const int i = ib + tid;
        const bool valid = i < (int)ktot;
        int s = 0, leaf = 0, len = 0, bs = 0;
        if (valid) {
            s = last_le(t.s_kb, nslots, i);
            leaf = i - t.s_kb[s];
            const int j = t.s_a0[s] + leaf;
            len = P.alen[j];
            bs = P.abs[j];
        }
        const bool ne = len > 0;
        long long tot;
        const long long ex = block_excl_scan<NT, long long>(
            ((long long)(ne ? 1 : 0) << 32) | (long long)len, ws, &tot);
        const int li = lcarry + (int)(ex >> 32);
        const int po = pcarry + (int)(ex & 0xffffffffLL);
        if (valid && leaf == 0)
            t.s_lb[s] = li;
        if (ne && li < kMidMaxLists) {
            t.loff[li] = po;
            t.lbs[li] = bs;
            t.lslot[li] = (unsigned char)s;
            t.lleaf[li] = (unsigned char)leaf;
        }
        lcarry += (int)(tot >> 32);
        pcarry += (int)(tot & 0xffffffffLL);
    }
    if (lcarry > kMidMaxLists || pcarry > kMidCap) {
        if (tid == 0)
            atomicOr(&P.cnt->err, kErrWindowOverflow);
        __syncthreads();
        return false;
    }
    if (tid == 0) {
        t.loff[lcarry] = pcarry;
        t.s_lb[nslots] = lcarry;
        t.misc[0] = nslots;
        t.misc[1] = lcarry;
        t.misc[2] = pcarry;
    }
    __syncthreads();
    return true;
}

// Batch bounds: rows [r0, r1) of batch b.
__device__ __forceinline__ void mid_bounds(const PlanDev &P, int M, int b, int nb, int &r0, int &r1)
{
    r0 = P.batch_start[b];
    r1 = (b + 1 < nb) ? P.batch_start[b + 1] : M;
}

// B positions of the batch products [p, p+n), n <= kGatherBatch, and their
// lists.  j/lbeg/lend/bsj carry the walk across calls.
__device__ __forceinline__ void mid_positions(const MidBatch &t, int p, int n, int &j, int &lbeg,
                                              int &lend, int &bsj, int (&addr)[kGatherBatch],
                                              int (&lid)[kGatherBatch])
{
#pragma unroll
    for (int i = 0; i < kGatherBatch; i++) {
        if (i < n) {
            while (p + i >= lend) {
                j++;
                lbeg = lend;
                lend = t.loff[j + 1];
                bsj = t.lbs[j];
            }
            addr[i] = bsj + (p + i - lbeg);
            lid[i] = j;
        }
    }
}

// ---------------------------------------------------------------------------
// Symbolic: exact nnz of every mid row by shared-memory hashing.
// ---------------------------------------------------------------------------
template <int UNUSED = 0>
__global__ void __launch_bounds__(kMidThreads) k_mid_symbolic(CsrDev A, CsrDev B, PlanDev P)
{
    constexpr int NT = kMidThreads;
    using L = MidSymLayout;
    extern __shared__ __align__(16) unsigned char smem[];
    int *tab = (int *)(smem + L::o_tab);
    int *hbase = (int *)(smem + L::o_hbase);
    int *cnt = (int *)(smem + L::o_cnt);
    long long *ws = (long long *)(smem + L::o_ws);
    MidBatch t = mid_tables<int, L>(smem);
    const int tid = threadIdx.x;
    const int M = A.M;
    const int nb = P.cnt->n_batch;
    const int *__restrict__ bcol = B.col;
    for (;;) {
        if (tid == 0)
            t.misc[4] = atomicAdd(&P.cnt->work_bsym, 1);
        __syncthreads();
        const int b = t.misc[4];
        __syncthreads();
        if (b >= nb)
            break;
        int r0, r1;
        mid_bounds(P, M, b, nb, r0, r1);
        if (!mid_setup(A, P, r0, r1, t, ws))
            continue;
        const int nslots = t.misc[0], nlists = t.misc[1], nprod = t.misc[2];
        // per-row hash regions: a power of two >= 1.5 * products
        int hs = 0;
        if (tid < nslots) {
            const int f = t.loff[t.s_lb[tid + 1]] - t.loff[t.s_lb[tid]];
            const int want = f + (f >> 1) + 1;
            hs = 32;
            while (hs < want)
                hs <<= 1;
            cnt[tid] = 0;
        }
        long long htot;
        const int hb = (int)block_excl_scan<NT, long long>(hs, ws, &htot);
        if (tid < nslots)
            hbase[tid] = hb;
        if (tid == 0)
            hbase[nslots] = (int)htot;
        const bool fits = htot <= kMidHashCap;
        for (int i = tid; i < (fits ? (int)htot : 0); i += NT)
            tab[i] = -1;
        __syncthreads();
        if (!fits) {
            if (tid == 0)
                atomicOr(&P.cnt->err, kErrWindowOverflow);
            continue;
        }
        const int ipt = (nprod + NT - 1) / NT;
        const int p0 = min(tid * ipt, nprod), p1 = min(p0 + ipt, nprod);
        if (p0 < p1) {
            int j = last_le(t.loff, nlists, p0);
            int lbeg = t.loff[j], lend = t.loff[j + 1], bsj = t.lbs[j];
            for (int p = p0; p < p1; p += kGatherBatch) {
                const int n = min(kGatherBatch, p1 - p);
                int addr[kGatherBatch], lid[kGatherBatch], c[kGatherBatch];
                mid_positions(t, p, n, j, lbeg, lend, bsj, addr, lid);
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++)
                    if (i < n)
                        c[i] = bcol[addr[i]];
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++) {
                    if (i < n) {
                        const int s = t.lslot[lid[i]];
                        const int base = hbase[s];
                        const int hsz = hbase[s + 1] - base;
                        const int sh = 32 - (31 - __clz(hsz));
                        unsigned h = ((unsigned)c[i] * 2654435761u) >> sh;
                        for (;;) {
                            const int old = atomicCAS(&tab[base + h], -1, c[i]);
                            if (old == -1) {
                                atomicAdd(&cnt[s], 1);
                                break;
                            }
                            if (old == c[i])
                                break;
                            h = (h + 1) & (unsigned)(hsz - 1);
                        }
                    }
                }
            }
        }
        __syncthreads();
        if (tid < nslots)
            P.nnz[t.s_row[tid]] = cnt[tid];
        __syncthreads();
    }
}

// One level of the bottom-up merge: runs are groups of 2^L consecutive lists
// of one slot; adjacent runs (2m, 2m+1) merge, a run without a right
// neighbour is copied.  Thread positions are [p0, p1) of the output.
__device__ __forceinline__ void mid_merge_level(int L, const unsigned short *__restrict__ src,
                                                unsigned short *__restrict__ dst,
                                                const int *__restrict__ col, const MidBatch &t,
                                                int nlists, int p0, int p1)
{
    if (p0 >= p1)
        return;
    int j = last_le(t.loff, nlists, p0);
    int p = p0;
    while (p < p1) {
        const int s = t.lslot[j];
        const int lb = t.s_lb[s], ns = t.s_lb[s + 1] - lb;
        const int pg = ((j - lb) >> L) & ~1;
        const int l0 = lb + (pg << L);
        const int l1 = lb + min((pg + 1) << L, ns);
        const int l2 = lb + min((pg + 2) << L, ns);
        const int ls = t.loff[l0], le = t.loff[l1], re = t.loff[l2];
        const int stop = min(p1, re);
        if (le == re) {
            // a run without a right neighbour is copied, unless it is the
            // slot's only run: a fully merged slot stays in the buffer of
            // its own last level (the readers pick it by the level parity)
            if (ns <= (1 << L))
                p = stop;
            for (; p < stop; p++)
                dst[p] = src[p];
        } else {
            const int na = le - ls, nb = re - le, d = p - ls;
            int lo = max(0, d - nb), hi = min(d, na);
            while (lo < hi) {
                const int m = (lo + hi) >> 1;
                if (col[src[ls + m]] <= col[src[le + d - 1 - m]])
                    lo = m + 1;
                else
                    hi = m;
            }
            int ia = lo, ib = d - lo;
            int ea = ia < na ? src[ls + ia] : 0;
            int eb = ib < nb ? src[le + ib] : 0;
            int ca = ia < na ? col[ea] : INT_MAX;
            int cb = ib < nb ? col[eb] : INT_MAX;
            for (; p < stop; p++) {
                if (ca <= cb) {
                    dst[p] = (unsigned short)ea;
                    if (++ia < na) {
                        ea = src[ls + ia];
                        ca = col[ea];
                    } else {
                        ca = INT_MAX;
                    }
                } else {
                    dst[p] = (unsigned short)eb;
                    if (++ib < nb) {
                        eb = src[le + ib];
                        cb = col[eb];
                    } else {
                        cb = INT_MAX;
                    }
                }
            }
        }
        j = l2;
    }
}

// ---------------------------------------------------------------------------
// Numeric: stable merge by column, order-exact reduction, ordered store.
// ---------------------------------------------------------------------------
// SCRATCH: the one-call Precise form runs this kernel before nnz(C) is
// known and writes each row at P.mid_pre[row] of a scratch pair (ccol, cval)
// sized by the batch weights, with its length in P.nnz; k_mid_compact moves
// the rows to C once crpt exists.
template <typename T, bool UPPER, bool SCRATCH = false>
__global__ void __launch_bounds__(kMidThreads) k_mid_numeric(CsrDev A, CsrDev B, PlanDev P,
                                                             const int *crpt, int *ccol, T *cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    constexpr int NT = kMidThreads;
    using L = MidNumLayout<T>;
    extern __shared__ __align__(16) unsigned char smem[];
    int *col = (int *)(smem + L::o_col);
    T *val = (T *)(smem + L::o_val);
    unsigned short *idx0 = (unsigned short *)(smem + L::o_idx0);
    unsigned short *idx1 = (unsigned short *)(smem + L::o_idx1);
    unsigned short *lidx = (unsigned short *)(smem + L::o_lidx);
    int *s_hb = (int *)(smem + L::o_shb);
    unsigned *head = (unsigned *)(smem + L::o_head);
    long long *ws = (long long *)(smem + L::o_ws);
    MidBatch t = mid_tables<T, L>(smem);
    const int tid = threadIdx.x;
    const int M = A.M;
    const int nb = P.cnt->n_batch;
    const T *__restrict__ aval = (const T *)A.val;
    const T *__restrict__ bval = (const T *)B.val;
    const int *__restrict__ bcol = B.col;
    for (;;) {
        if (tid == 0)
            t.misc[4] = atomicAdd(&P.cnt->work_bnum, 1);
        __syncthreads();
        const int b = t.misc[4];
        __syncthreads();
        if (b >= nb)
            break;
        int r0, r1;
        mid_bounds(P, M, b, nb, r0, r1);
        if (!mid_setup(A, P, r0, r1, t, ws))
            continue;
        const int nslots = t.misc[0], nlists = t.misc[1], nprod = t.misc[2];
        const int ipt = (nprod + NT - 1) / NT;
        const int p0 = min(tid * ipt, nprod), p1 = min(p0 + ipt, nprod);
        // stage products in list-major order (batched independent gathers)
        if (p0 < p1) {
            int j = last_le(t.loff, nlists, p0);
            int lbeg = t.loff[j], lend = t.loff[j + 1], bsj = t.lbs[j];
            for (int p = p0; p < p1; p += kGatherBatch) {
                const int n = min(kGatherBatch, p1 - p);
                int addr[kGatherBatch], lid[kGatherBatch], c[kGatherBatch];
                T bv[kGatherBatch], av[kGatherBatch];
                mid_positions(t, p, n, j, lbeg, lend, bsj, addr, lid);
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++) {
                    if (i < n) {
                        const bool in = BRM_IN(P.cnt, addr[i], B.nnz);
                        c[i] = in ? bcol[addr[i]] : 0;
                        bv[i] = in ? bval[addr[i]] : T(0);
                        av[i] = aval[t.s_a0[t.lslot[lid[i]]] + t.lleaf[lid[i]]];
                    }
                }
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++) {
                    if (i < n) {
                        const int e = p + i;
                        col[e] = c[i];
                        val[e] = vmul(av[i], bv[i]);
                        lidx[e] = (unsigned short)lid[i];
                        idx0[e] = (unsigned short)e;
                    }
                }
            }
        }
        for (int i = tid; i < (nprod + 31) / 32; i += NT)
            head[i] = 0;
        int lev = 0;
        if (tid < nslots)
            lev = ceil_log2(t.s_lb[tid + 1] - t.s_lb[tid]);
        const int levels = (int)block_max<NT, long long>(lev, ws);
        {
            unsigned short *src = idx0, *dst = idx1;
            for (int lv = 0; lv < levels; lv++) {
                mid_merge_level(lv, src, dst, col, t, nlists, p0, p1);
                __syncthreads();
                unsigned short *x = src;
                src = dst;
                dst = x;
            }
        }
        // A slot with n lists ends its merge after ceil_log2(n) levels, in
        // idx1 when that count is odd and in idx0 when it is even.  Each
        // thread walks its positions [p0, p1) slot by slot.
        int s_cur = -1, s_beg = 0, s_end = 0;
        const unsigned short *sb = idx0;
        auto enter = [&](int p) {
            while (p >= s_end) {
                s_cur = s_cur < 0 ? t.lslot[last_le(t.loff, nlists, p)] : s_cur + 1;
                s_beg = t.loff[t.s_lb[s_cur]];
                s_end = t.loff[t.s_lb[s_cur + 1]];
                sb = (ceil_log2(t.s_lb[s_cur + 1] - t.s_lb[s_cur]) & 1) ? idx1 : idx0;
            }
        };
        // heads: first product of each (row, column) run
        int nh = 0;
        {
            int prev_c = 0;
            for (int p = p0; p < p1; p++) {
                enter(p);
                const int c = col[sb[p]];
                if (p == p0 && p > s_beg)
                    prev_c = col[sb[p - 1]];
                if (p == s_beg || c != prev_c) {
                    atomicOr(&head[p >> 5], 1u << (p & 31));
                    nh++;
                }
                prev_c = c;
            }
        }
        long long htot;
        int hx = (int)block_excl_scan<NT, long long>(nh, ws, &htot);
        // head index of each slot's first position
        {
            int h = hx;
            s_cur = -1;
            s_end = 0;
            for (int p = p0; p < p1; p++) {
                if ((head[p >> 5] >> (p & 31)) & 1u) {
                    enter(p);
                    if (p == s_beg)
                        s_hb[s_cur] = h;
                    h++;
                }
            }
            if (tid == 0)
                s_hb[nslots] = (int)htot;
        }
        __syncthreads();
        // one thread per head: reduce its run (in leaf order: the merge is
        // stable) and store it
        {
            int h = hx;
            s_cur = -1;
            s_end = 0;
            for (int p = p0; p < p1; p++) {
                if (!((head[p >> 5] >> (p & 31)) & 1u))
                    continue;
                enter(p);
                const int e = sb[p];
                const int row = t.s_row[s_cur];
                const long long base = SCRATCH ? P.mid_pre[row]
                                       : (UPPER ? P.scan_flop[row] : (long long)crpt[row]);
                const long long o = base + (h - s_hb[s_cur]);
                int q = p + 1;
                T v = val[e];
                if (q < s_end && !((head[q >> 5] >> (q & 31)) & 1u)) {
                    const int e1 = sb[q++];
                    if (!(q < s_end && !((head[q >> 5] >> (q & 31)) & 1u))) {
                        v = vadd(v, val[e1]);  // two leaves: left + right
                    } else {
                        // leaves < 256: at most 8 stack entries below the top
                        RegShiftReduce<T, 9> sr;
                        sr.init(t.lleaf[lidx[e]], v);
                        sr.push(t.lleaf[lidx[e1]], val[e1]);
                        for (; q < s_end && !((head[q >> 5] >> (q & 31)) & 1u); q++) {
                            const int e2 = sb[q];
                            sr.push(t.lleaf[lidx[e2]], val[e2]);
                        }
                        v = sr.finish();
                    }
                }
                if (BRM_IN(P.cnt, o, SCRATCH ? P.mid_cap : P.c_cap)) {
                    ccol[o] = col[e];
                    cval[o] = v;
                }
                h++;
            }
        }
        if (tid < nslots) {
            const int row = t.s_row[tid];
            const int len = s_hb[tid + 1] - s_hb[tid];
            if (UPPER || SCRATCH)
                P.nnz[row] = len;
            else if (len != crpt[row + 1] - crpt[row])
                atomicOr(&P.cnt->err, kErrNnzMismatch);
        }
        __syncthreads();
    }
}

// Batch starts: batch b begins at the first row whose mid-weight prefix is
// >= b * W; n_batch = ceil(total / W), W = P.mid_limit (<= kMidFlop, every
// mid row weighs at most W, so a batch weighs less than 2 W <= kMidCap).
template <int UNUSED = 0>
__global__ void __launch_bounds__(256) k_batch_starts(PlanDev P, int M)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r > M)
        return;
    const long long W = P.mid_limit;
    const long long hi = P.mid_pre[r];
    const long long lo = r > 0 ? P.mid_pre[r - 1] : -1;
    const long long b = hi / W;
    if (b * W > lo && b <= M)
        P.batch_start[b] = r;
    if (r == M)
        P.cnt->n_batch = (int)((hi + W - 1) / W);
}

// Moves the mid rows written by k_mid_numeric<..., SCRATCH> (row at
// P.mid_pre[row]) and k_mid_warp<..., kMwScratch> (row at P.mid_pre[M] +
// P.mw_pre[row]), P.nnz[row] entries each, from the scratch to C at
// crpt[row].  One warp per row; rows that are not mid rows are skipped.
template <typename T>
__global__ void __launch_bounds__(256) k_mid_compact(PlanDev P, int M, const int *__restrict__ scol,
                                                     const T *__restrict__ sval, const int *crpt,
                                                     int *__restrict__ ccol, T *__restrict__ cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int r1 = min(M, P.r_hi);
    // warp and group rows from their row lists, then (only when there are
    // batches) the batched mid rows by a sweep over the rows
    const int nw1 = P.cnt->bin_count[kBinMidWarp];
    const int nw4 = P.cnt->bin_count[kBinMidGroup];
    const int nwt = P.cnt->bin_count[kBinMidTile];
    const int nwt2 = P.cnt->bin_count[kBinMidTile2];
    const int nw5 = P.cnt->bin_count[kBinMidGroup2];
    const int nlist = nw1 + nw4 + nwt + nwt2 + nw5;
    const int nsweep = P.cnt->n_batch > 0 ? r1 - P.r_lo : 0;
    for (int it = gw; it < nlist + nsweep; it += nwarps) {
        int row;
        long long src;
        if (it < nlist) {
            row = it < nw1              ? P.rows[(size_t)kBinMidWarp * M + it]
                  : it < nw1 + nw4       ? P.rows[(size_t)kBinMidGroup * M + (it - nw1)]
                  : it < nw1 + nw4 + nwt ? P.rows[(size_t)kBinMidTile * M + (it - nw1 - nw4)]
                  : it < nw1 + nw4 + nwt + nwt2
                      ? P.rows[(size_t)kBinMidTile2 * M + (it - nw1 - nw4 - nwt)]
                      : P.rows[(size_t)kBinMidGroup2 * M + (it - nw1 - nw4 - nwt - nwt2)];
            if (row < P.r_lo || row >= r1)
                continue;
            src = P.mid_pre[M] + P.mw_pre[row];
        } else {
            row = P.r_lo + (it - nlist);
            if (P.mid_flop[row] == 0)
                continue;
            src = P.mid_pre[row];
        }
        const long long dst = crpt[row];
        int n = P.nnz[row];
        if (n > 0 && !(BRM_IN(P.cnt, dst + n - 1, P.c_cap) && BRM_IN(P.cnt, src + n - 1, P.mid_cap)))
            n = 0;  // checked build: a row outside C or the scratch is skipped
        // four elements per lane in flight before the stores
        int i = lane;
        for (; i + 96 < n; i += 128) {
            int c[4];
            T v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                c[u] = scol[src + i + 32 * u];
                v[u] = sval[src + i + 32 * u];
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                ccol[dst + i + 32 * u] = c[u];
                cval[dst + i + 32 * u] = v[u];
            }
        }
        for (; i < n; i += 32) {
            ccol[dst + i] = scol[src + i];
            cval[dst + i] = sval[src + i];
        }
    }
}

}  // namespace brm
