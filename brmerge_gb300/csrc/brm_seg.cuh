// brm_seg.cuh -- segmented processing of heavy rows.
//
// A heavy row (more products or lists than a mid-row batch holds) is cut into
// column segments [c_lo, c_hi).  Columns of C are independent, so the merge
// tree of the row restricted to a column range is the same tree with every
// list restricted to that range (BRMerge-SpGEMM/inc/spgemm.h:639-707): the
// leaf index of a product, and therefore the order of its additions, does
// not depend on the cut.  Three steps:
//
//   1. planning (symbolic phase, one CTA per heavy row, longest rows first):
//      a bitmap of the row's columns and a product count per 128-column group
//      over chunks of kPlanBits columns give the row's exact nnz and the cut
//      points: a cut before group g when the running product count crosses a
//      multiple of the cut target (at most kSegCut, a runtime knob) and
//      around groups holding more than kSegCap minus the target (inside such
//      a group the cuts are per column, from 16-bit per-column counts); a
//      segment then holds <= kSegCap products.  Its
//      output offset within the row (distinct columns before c_lo) comes
//      from the same bitmap.
//   2. split table (numeric phase): for every segment boundary and every list
//      of the row, the first list position at or after the boundary column
//      (one block per boundary, one binary search per list).
//   3. segment kernel (numeric phase, one CTA pass per segment): stage the
//      segment's products in list-major order; the rank u of every product's
//      column among the segment's distinct columns comes from a two-level
//      bitmap (a summary bit per nonempty 32-column word, then the compressed
//      words); a counting sort on u groups each column's contributions; one
//      thread per output column puts up to eight of them in leaf order in
//      registers and evaluates the merge tree (closed forms for three and
//      four, a register ShiftReduce up to eight); longer columns are ranked
//      by leaf by a warp and handed to the column reducer (step 4).  Column u
//      is stored at position u of the row's segment (coalesced).
//   4. column reducer: one thread per long column, ShiftReduce with the
//      stack in registers over the leaf-ordered products.
#pragma once

#include <climits>

#include "brm_check.cuh"
#include "brm_common.cuh"
#include "brm_mid.cuh"
#include "brm_plan.h"

namespace brm {

constexpr int kPlanThreads = 512;
// Segment cuts are placed at planning-group boundaries (kPlanGroupBits
// columns); a dense group (more than kSegCap - cut products) is a segment of
// its own, and one above kSegCap products gets per-column counts and is cut
// inside (at most kDenseGroups such groups per chunk).
constexpr int kPlanGroupLog2 = 7;
constexpr int kPlanGroupBits = 1 << kPlanGroupLog2;      // 128 columns
constexpr int kPlanGroupWords = kPlanGroupBits / 32;     // 4 bitmap words
constexpr int kPlanGroups = kPlanBits / kPlanGroupBits;  // 2048 per chunk
constexpr int kDenseGroups = 128;  // 16-bit column counts: a count is at most k <= 65535

struct PlanLayout {
    static constexpr size_t o_bm = 0;
    static constexpr size_t o_hist = o_bm + kPlanWords * 4;
    static constexpr size_t o_gpop = o_hist + kPlanGroups * 4;
    static constexpr size_t o_dix = o_gpop + kPlanGroups * 2;
    static constexpr size_t o_ccnt = o_dix + kPlanGroups * 2;
    static constexpr size_t o_lst = o_ccnt + kDenseGroups * kPlanGroupBits * 2;
    static constexpr size_t o_loffs = o_lst + (kPlanThreads + 1) * 4;
    static constexpr size_t o_ws = o_loffs + (kPlanThreads + 1) * 4 + 8;
    static constexpr size_t o_misc = o_ws + (kPlanThreads / 32 + 1) * 8;
    static constexpr size_t bytes = o_misc + 64;
};

// Calls f(rc) for every product of the row, rc = column - base; with clip,
// only for the products whose column lies in [lo, chi) (each list is cut by
// binary search).  The products are split evenly over the block: the lists
// are taken NT at a time, their lengths scanned, and every thread walks a
// contiguous share of the chunk's products (a single very long list of a
// power-law row is shared by all threads instead of one group).  A thread
// sees its products in list order, column-sorted within each list.
// lst/loffs are NT+1 ints of shared scratch.
template <int NT, typename Fn>
__device__ __forceinline__ void plan_products(const PlanDev &P, const int *__restrict__ bcol,
                                              int a0, int k, bool clip, int lo, int chi, int base,
                                              int *lst, int *loffs, long long *ws, Fn f)
{
    const int tid = threadIdx.x;
    for (int lb = 0; lb < k; lb += NT) {
        const int l = lb + tid;
        int s = 0, len = 0;
        if (l < k) {
            len = P.alen[a0 + l];
            s = P.abs[a0 + l];
            if (clip && len > 0) {
                int e = s + len;
                s = lower_bound_idx(bcol, s, e, lo);
                e = lower_bound_idx(bcol, s, e, chi);
                len = e - s;
            }
        }
        long long tot;
        const int off = (int)block_excl_scan<NT, long long>(len, ws, &tot);
        lst[tid] = s;
        loffs[tid] = off;
        if (tid == 0)
            loffs[NT] = (int)tot;
        __syncthreads();
        const int n = (int)tot;
        const int ipt = (n + NT - 1) / NT;
        const int p0 = min(tid * ipt, n), p1 = min(p0 + ipt, n);
        if (p0 < p1) {
            int j = last_le(loffs, NT, p0);
            int lbeg = loffs[j], lend = loffs[j + 1], bsj = lst[j];
            for (int p = p0; p < p1; p += kGatherBatch) {
                const int m = min(kGatherBatch, p1 - p);
                int addr[kGatherBatch], c[kGatherBatch];
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++) {
                    if (i < m) {
                        while (p + i >= lend) {
                            j++;
                            lbeg = lend;
                            lend = loffs[j + 1];
                            bsj = lst[j];
                        }
                        addr[i] = bsj + (p + i - lbeg);
                    }
                }
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++)
                    c[i] = i < m ? bcol[addr[i]] : 0;
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++)
                    if (i < m)
                        f(c[i] - base);
            }
        }
        __syncthreads();
    }
}

// Walks the segment starts of planning group g (chunk-relative) in column
// order and calls f(column_in_group, product_prefix, distinct_prefix) for
// each.  `run` packs (products << 32 | distinct columns) before group g and
// ph is the product count of group g-1.  A dense group (more than
// dense = kSegCap - cut products) is always cut before and after; it is one
// segment when it holds at most kSegCap products, and inside a larger one a
// new segment starts at a column when the running product count would exceed
// `cut` (a single column above `cut` is a segment of its own).  Any other
// group starts a segment when the group before it crossed a multiple of
// `cut`, so a segment holds less than cut + dense = kSegCap products.
template <typename Fn>
__device__ __forceinline__ void plan_group_starts(int g, unsigned h, unsigned ph,
                                                  unsigned long long run,
                                                  const unsigned short *ccnt, unsigned cut,
                                                  unsigned dense, Fn f)
{
    const unsigned pe = (unsigned)(run >> 32);
    const unsigned ue = (unsigned)(run & 0xffffffffu);
    if (h > dense && h <= (unsigned)kSegCap) {
        f(0, pe, ue);
        return;
    }
    if (h > dense) {
        f(0, pe, ue);
        unsigned acc = 0, pp = pe, uu = ue;
        for (int c = 0; c < kPlanGroupBits; c++) {
            const unsigned cc = ccnt[c];
            if (cc == 0)
                continue;
            if (acc > 0 && acc + cc > cut) {
                f(c, pp, uu);
                acc = 0;
            }
            acc += cc;
            pp += cc;
            uu++;  // a column with products is one distinct column
        }
        return;
    }
    const bool start = (g == 0) || ph > dense || (pe / cut) != ((pe - ph) / cut);
    if (start)
        f(0, pe, ue);
}

// ---------------------------------------------------------------------------
// 1. planning
// ---------------------------------------------------------------------------
template <int UNUSED = 0>
__global__ void __launch_bounds__(kPlanThreads) k_heavy_plan(CsrDev A, CsrDev B, PlanDev P)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    constexpr int NT = kPlanThreads;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned *bm = (unsigned *)(smem + PlanLayout::o_bm);
    unsigned *hist = (unsigned *)(smem + PlanLayout::o_hist);
    unsigned short *gpop = (unsigned short *)(smem + PlanLayout::o_gpop);
    unsigned short *dix = (unsigned short *)(smem + PlanLayout::o_dix);
    // per-column product counts of groups above kSegCap products, two 16-bit
    // counters a word
    unsigned *ccnt2 = (unsigned *)(smem + PlanLayout::o_ccnt);
    const unsigned short *ccnt = (const unsigned short *)(smem + PlanLayout::o_ccnt);
    int *lst = (int *)(smem + PlanLayout::o_lst);
    int *loffs = (int *)(smem + PlanLayout::o_loffs);
    long long *ws = (long long *)(smem + PlanLayout::o_ws);
    int *misc = (int *)(smem + PlanLayout::o_misc);
    const int tid = threadIdx.x;
    const int M = A.M;
    // rows above kHugeFlop products sit at the end of the list; take them first
    const int nhuge = P.cnt->n_huge;
    const int nrows = P.cnt->bin_count[kBinHeavy] + nhuge;
    const int *rows = P.rows + (size_t)kBinHeavy * M;
    const int *__restrict__ bcol = B.col;
    const unsigned cut = (unsigned)P.seg_cut;                // <= kSegMaxCut
    const unsigned dense = (unsigned)(kSegCap - P.seg_cut);  // >= kSegCap / 4
    for (int i = tid; i < kPlanWords; i += NT)
        bm[i] = 0;
    for (int i = tid; i < kPlanGroups; i += NT)
        hist[i] = 0;
    for (;;) {
        if (tid == 0)
            misc[0] = atomicAdd(&P.cnt->work_plan, 1);
        __syncthreads();
        const int item = misc[0];
        __syncthreads();
        if (item >= nrows)
            break;
        const int row = item < nhuge ? rows[M - 1 - item] : rows[item - nhuge];
        const int a0 = A.rpt[row];
        const int k = A.rpt[row + 1] - a0;
        const long long F = P.flop[row];
        const unsigned long long base = P.seg_base[row];
        const unsigned long long bound = seg_bound(F, B.N, P.seg_cut);
        const int2 cr = P.crange[row];  // written by the analysis
        const int mn = cr.x, mx = cr.y;
        if (mx < 0 || mn < 0 || mx >= B.N) {
            if (tid == 0) {
                if (mx >= 0)
                    atomicOr(&P.cnt->err, kErrBadInput);
                P.nnz[row] = 0;
                P.seg_n[row] = 0;
            }
            continue;
        }
        const bool multi = (long long)mx + 1 - mn > kPlanBits;
        long long u_run = 0;
        int nseg = 0;
        bool fail = false;
        for (long long clo = mn; clo <= mx; clo += kPlanBits) {
            const int lo = (int)clo;
            const int chi = (int)min((long long)mx + 1, clo + kPlanBits);
            const int span = chi - lo;
            const int ng = (span + kPlanGroupBits - 1) >> kPlanGroupLog2;
            // bm and hist are zero here: cleared at the start and after every chunk
            if (tid == 0) {
                misc[4] = INT_MAX;  // first group cut per column
                misc[5] = -1;       // last group cut per column
            }
            __syncthreads();
            // pass over the chunk's products: column bitmap and products per
            // group.  A thread's products are column-sorted within each list,
            // so runs in one word (group) are gathered in registers and
            // flushed once.
            bool bad = false;
            unsigned run_w = 0xffffffffu, run_b = 0, run_g = 0xffffffffu, run_n = 0;
            plan_products<NT>(P, bcol, a0, k, multi, lo, chi, lo, lst, loffs, ws, [&](int rc) {
                if ((unsigned)rc >= (unsigned)span) {
                    bad = true;
                    return;
                }
                const unsigned w = (unsigned)rc >> 5;
                if (w != run_w) {
                    if (run_b)
                        atomicOr(&bm[run_w], run_b);
                    run_w = w;
                    run_b = 0;
                }
                run_b |= 1u << (rc & 31);
                const unsigned g = (unsigned)rc >> kPlanGroupLog2;
                if (g != run_g) {
                    if (run_n)
                        atomicAdd(&hist[run_g], run_n);
                    run_g = g;
                    run_n = 0;
                }
                run_n++;
            });
            if (run_b)
                atomicOr(&bm[run_w], run_b);
            if (run_n)
                atomicAdd(&hist[run_g], run_n);
            if (bad)
                atomicOr(&P.cnt->err, kErrBadInput);
            __syncthreads();
            const int gpt = (ng + NT - 1) / NT;
            const int g0 = min(tid * gpt, ng), g1 = min(g0 + gpt, ng);
            // distinct columns per group; groups above kSegCap products get
            // per-column counts
            int nd_local = 0, dlo = INT_MAX, dhi = -1;
            unsigned long long sp = 0;
            for (int g = g0; g < g1; g++) {
                const unsigned h = hist[g];
                int pc = 0;
#pragma unroll
                for (int q = 0; q < kPlanGroupWords; q++)
                    pc += __popc(bm[g * kPlanGroupWords + q]);
                gpop[g] = (unsigned short)pc;
                if (h > (unsigned)kSegCap) {
                    nd_local++;
                    dlo = min(dlo, g);
                    dhi = g;
                }
                sp += ((unsigned long long)h << 32) | (unsigned)pc;
            }
            if (nd_local) {
                atomicMin(&misc[4], dlo);
                atomicMax(&misc[5], dhi);
            }
            long long ndt;
            int dx = (int)block_excl_scan<NT, long long>(nd_local, ws, &ndt);
            const int nd = (int)ndt;
            if (nd > kDenseGroups)
                fail = true;  // uniform
            if (!fail && nd > 0) {
                for (int g = g0; g < g1; g++)
                    if (hist[g] > (unsigned)kSegCap)
                        dix[g] = (unsigned short)dx++;
                for (int i = tid; i < nd * kPlanGroupBits / 2; i += NT)
                    ccnt2[i] = 0;
                __syncthreads();
                // only the columns from the first to the last such group
                const int dlo_c = lo + kPlanGroupBits * misc[4];
                const int dhi_c = (int)min((long long)chi,
                                           (long long)lo + (long long)kPlanGroupBits * (misc[5] + 1));
                plan_products<NT>(P, bcol, a0, k, true, dlo_c, dhi_c, lo, lst, loffs, ws, [&](int rc) {
                    if ((unsigned)rc < (unsigned)span) {
                        const int g = rc >> kPlanGroupLog2;
                        if (hist[g] > (unsigned)kSegCap) {
                            const int slot = dix[g] * kPlanGroupBits + (rc & (kPlanGroupBits - 1));
                            atomicAdd(&ccnt2[slot >> 1], 1u << (16 * (slot & 1)));
                        }
                    }
                });
                bool big = false;
                for (int i = tid; i < nd * kPlanGroupBits; i += NT)
                    big |= ccnt[i] > kSegCap;
                fail = __syncthreads_or(big) != 0;
            }
            long long tot;
            const unsigned long long ex = (unsigned long long)block_excl_scan<NT, long long>(
                (long long)sp, ws, &tot);
            // count the chunk's segment starts
            int nstart = 0;
            if (!fail) {
                unsigned long long run = ex;
                unsigned ph = (g0 > 0 && g0 < ng) ? hist[g0 - 1] : 0u;
                for (int g = g0; g < g1; g++) {
                    const unsigned h = hist[g];
                    plan_group_starts(g, h, ph, run,
                                      h > (unsigned)kSegCap ? ccnt + dix[g] * kPlanGroupBits : ccnt, cut,
                                      dense, [&](int, unsigned, unsigned) { nstart++; });
                    run += ((unsigned long long)h << 32) | (unsigned)gpop[g];
                    ph = h;
                }
            }
            long long stot;
            const int sx = (int)block_excl_scan<NT, long long>(nstart, ws, &stot);
            if ((unsigned long long)(nseg + stot) > bound)
                fail = true;
            const long long u_chunk = u_run;
            u_run += (long long)((unsigned long long)tot & 0xffffffffull);
            if (fail) {
                __syncthreads();
                for (int g = g0; g < g1; g++) {
                    hist[g] = 0;
#pragma unroll
                    for (int q = 0; q < kPlanGroupWords; q++)
                        bm[g * kPlanGroupWords + q] = 0;
                }
                __syncthreads();
                continue;  // keep counting distinct columns; the row takes the spill path
            }
            // write the chunk's segments: c_lo, u_off and the product prefix
            {
                unsigned long long run = ex;
                unsigned ph = (g0 > 0 && g0 < ng) ? hist[g0 - 1] : 0u;
                int r = sx;
                for (int g = g0; g < g1; g++) {
                    const unsigned h = hist[g];
                    plan_group_starts(g, h, ph, run,
                                      h > (unsigned)kSegCap ? ccnt + dix[g] * kPlanGroupBits : ccnt, cut,
                                      dense, [&](int c, unsigned pe, unsigned ue) {
                                          if (BRM_IN(P.cnt, base + nseg + r, P.cnt->seg_cap)) {
                                              SegDesc &d = P.seg[base + nseg + r];
                                              d.row = row;
                                              d.c_lo = lo + kPlanGroupBits * g + c;
                                              d.u_off = (int)(u_chunk + (long long)ue);
                                              d.bidx = nseg + r;
                                              d.nprod = (int)pe;  // prefix; a count below
                                          }
                                          r++;
                                      });
                    run += ((unsigned long long)h << 32) | (unsigned)gpop[g];
                    ph = h;
                }
            }
            __syncthreads();  // descriptors of this chunk visible to the block
            for (int g = g0; g < g1; g++) {
                hist[g] = 0;
#pragma unroll
                for (int q = 0; q < kPlanGroupWords; q++)
                    bm[g * kPlanGroupWords + q] = 0;
            }
            // c_hi and product count of each segment: read every neighbour
            // first, then write (rounds of NT segments)
            const int ctot_prod = (int)((unsigned long long)tot >> 32);
            for (int i0 = 0; i0 < (int)stot; i0 += NT) {
                const int i = i0 + tid;
                int nc = 0, np = 0;
                if (i < (int)stot) {
                    const bool last = i + 1 == (int)stot;
                    nc = last ? chi : P.seg[base + nseg + i + 1].c_lo;
                    np = (last ? ctot_prod : P.seg[base + nseg + i + 1].nprod) -
                         P.seg[base + nseg + i].nprod;
                }
                __syncthreads();
                if (i < (int)stot) {
                    P.seg[base + nseg + i].c_hi = nc;
                    P.seg[base + nseg + i].nprod = np;
                }
                __syncthreads();
            }
            nseg += (int)stot;
        }
        if (tid == 0) {
            if (fail) {
                // a column denser than a segment holds, or too many cuts:
                // replay the merge for this row in global scratch (spill path)
                P.seg_n[row] = 0;
                P.spill[row] = 1;
                const int idx = atomicAdd(&P.cnt->spill_count, 1);
                P.spill_rows[idx] = row;
                P.spill_off[idx] = atomicAdd(&P.cnt->spill_bytes, spill_row_bytes(F, k));
                misc[1] = 0;
            } else {
                P.seg_n[row] = nseg;
                const unsigned long long tab =
                    atomicAdd(&P.cnt->table_cap, (unsigned long long)(nseg + 1) * (unsigned long long)k);
                misc[2] = (int)(tab & 0xffffffffull);
                misc[3] = (int)(tab >> 32);
                misc[1] = atomicAdd(&P.cnt->n_seg, nseg);
            }
            P.nnz[row] = (int)u_run;
        }
        __syncthreads();
        if (!fail) {
            const long long tab =
                (long long)(((unsigned long long)(unsigned)misc[3] << 32) | (unsigned)misc[2]);
            const int lpos = misc[1];
            for (int i = tid; i < nseg; i += NT) {
                if (BRM_IN(P.cnt, base + i, P.cnt->seg_cap) &&
                    BRM_IN(P.cnt, lpos + i, P.cnt->seg_cap)) {
                    P.seg[base + i].tab = tab;
                    P.seg_list[lpos + i] = (int)(base + i);
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// 2. split table: split[tab + b*k + l] = first position of list l at or after
//    boundary b (b = 0 .. nseg; boundary nseg is the end of the row).  One
//    block per segment computes its boundary's row of the table.
// ---------------------------------------------------------------------------
template <int UNUSED = 0>
__global__ void __launch_bounds__(256) k_split(CsrDev A, CsrDev B, PlanDev P)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    const int i0 = P.seg_range ? P.seg_range[0] : 0;
    const int nsegs = P.seg_range ? P.seg_range[1] : P.cnt->n_seg;
    const int *__restrict__ bcol = B.col;
    for (int it = i0 + blockIdx.x; it < nsegs; it += gridDim.x) {
        const int slot = P.seg_list[it];
        const int row = P.seg[slot].row;
        const int b = P.seg[slot].bidx;
        const int c_lo = P.seg[slot].c_lo;
        const long long tab = P.seg[slot].tab;
        const int nseg = P.seg_n[row];
        const int a0 = A.rpt[row];
        const int k = A.rpt[row + 1] - a0;
        int *t0 = P.split + tab + (long long)b * k;
        if (threadIdx.x == 0) {
            SegRun r;
            r.sp = tab + (long long)b * k;
            r.row = row;
            r.c_lo = c_lo;
            r.c_hi = P.seg[slot].c_hi;
            r.u_off = P.seg[slot].u_off;
            r.nprod = P.seg[slot].nprod;
            r.a0 = a0;
            r.k = k;
            r.next_u = (b + 1 < nseg) ? P.seg[slot + 1].u_off : P.nnz[row];
            P.run[it] = r;
        }
        for (int l = threadIdx.x; l < k; l += blockDim.x) {
            const int s = P.abs[a0 + l];
            const int e = s + P.alen[a0 + l];
            if (BRM_IN(P.cnt, tab + (long long)b * k + l, P.cnt->table_cap))
                t0[l] = (b == 0) ? s : lower_bound_idx(bcol, s, e, c_lo);
            if (b == nseg - 1 && BRM_IN(P.cnt, tab + (long long)(b + 1) * k + l, P.cnt->table_cap))
                t0[k + l] = e;
        }
    }
}

// ---------------------------------------------------------------------------
// 3. segment kernel
// ---------------------------------------------------------------------------
constexpr int kLongMin = 9;  // columns with this many products are reduced by warps
constexpr int kLongMax = kSegCap / kLongMin + 1;
constexpr int kSegPWords = kSegCap / 32;  // words of a bitmap over a segment's products
static_assert(kSegCap % 32 == 0 && kSegPWords <= 96, "p-bitmap prefix: three words per lane");

// Copies a segment record (48 bytes) into shared memory with cp.async.
__device__ __forceinline__ void copy_seg_run(SegRun *dst, const SegRun *src)
{
#pragma unroll
    for (int q = 0; q < 3; q++)
        cp_async16((unsigned char *)dst + 16 * q, (const unsigned char *)src + 16 * q);
}

template <typename T>
struct SegLayout {
    static constexpr int NW = kSegThreads / 32;
    static constexpr size_t o_loff = 0;
    static constexpr size_t o_lbs = o_loff + mid_a16((kSegCap + 1) * 4);
    static constexpr size_t o_lleaf = o_lbs + mid_a16(kSegCap * 4);
    static constexpr size_t o_prc = o_lleaf + mid_a16(kSegCap * 2);
    static constexpr size_t o_pval = o_prc + mid_a16(kSegCap * 4);
    static constexpr size_t o_pleaf = o_pval + mid_a16(kSegCap * sizeof(T));
    static constexpr size_t o_pu = o_pleaf + mid_a16(kSegCap * 2);
    static constexpr size_t o_ia = o_pu + mid_a16(kSegCap * 2);
    static constexpr size_t o_ib = o_ia + mid_a16(kSegCap * 2);
    // the summary words of a wide segment and their ranks are dead before
    // the scatter first writes ib, so they share its space
    static constexpr size_t o_summ = o_ib;
    static constexpr size_t o_srank = o_summ + mid_a16(kSumWords * 4);
    static_assert(kSumWords * 4 + kSumWords * 2 <= kSegCap * 2, "summary words fit in ib");
    static constexpr size_t o_cw = o_ib + mid_a16(kSegCap * 2);
    static constexpr size_t o_cwr = o_cw + mid_a16(kSegCap * 4);
    static constexpr size_t o_long = o_cwr + mid_a16((kSegCap + 1) * 2);
    static constexpr size_t o_ws = o_long + mid_a16(kLongMax * 2);
    static constexpr size_t o_misc = o_ws + mid_a16((NW + 1) * 8);
    static constexpr size_t o_run = o_misc + 64;  // the next segment's record
    static constexpr size_t bytes = o_run + sizeof(SegRun);
    // per-warp p-bitmaps and their word prefixes live in cw once u is known
    static_assert(NW * kSegPWords * 6 <= kSegCap * 4, "cw region holds the warp bitmaps");
};

template <typename T, bool UPPER>
__global__ void __launch_bounds__(kSegThreads, 512 / kSegThreads) k_seg_numeric(CsrDev A, CsrDev B, PlanDev P,
                                                             const int *crpt, int *ccol, T *cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    constexpr int NT = kSegThreads;
    using L = SegLayout<T>;
    extern __shared__ __align__(16) unsigned char smem[];
    int *loff = (int *)(smem + L::o_loff);
    int *ucnt = loff;  // per-column counts, then column starts (after staging)
    int *lbs = (int *)(smem + L::o_lbs);
    unsigned short *lleaf = (unsigned short *)(smem + L::o_lleaf);
    int *prc = (int *)(smem + L::o_prc);
    T *pval = (T *)(smem + L::o_pval);
    unsigned short *pleaf = (unsigned short *)(smem + L::o_pleaf);
    unsigned short *pu = (unsigned short *)(smem + L::o_pu);
    unsigned short *ia = (unsigned short *)(smem + L::o_ia);
    unsigned short *ib = (unsigned short *)(smem + L::o_ib);
    unsigned *summ = (unsigned *)(smem + L::o_summ);
    unsigned short *srank = (unsigned short *)(smem + L::o_srank);
    unsigned *cw = (unsigned *)(smem + L::o_cw);
    unsigned short *cwr = (unsigned short *)(smem + L::o_cwr);
    unsigned short *longu = (unsigned short *)(smem + L::o_long);
    long long *ws = (long long *)(smem + L::o_ws);
    int *wsi = (int *)(smem + L::o_ws);
    int *misc = (int *)(smem + L::o_misc);
    SegRun *srun = (SegRun *)(smem + L::o_run);
    const int tid = threadIdx.x;
    const int i0 = P.seg_range ? P.seg_range[0] : 0;
    const int nsegs = P.seg_range ? P.seg_range[1] : P.cnt->n_seg;
    const int *__restrict__ bcol = B.col;
    const T *__restrict__ bval = (const T *)B.val;
    const T *__restrict__ aval = (const T *)A.val;
    // thread 0 takes the next work item one segment ahead and copies its
    // record into srun (cp.async) while the current segment runs, so a
    // segment starts without a chain of dependent global loads
    int pf = 0;
    bool pf_copied = false;
    if (tid == 0)
        pf = i0 + atomicAdd(&P.cnt->work_seg, 1);
    for (;;) {
        if (tid == 0) {
            if (!pf_copied && pf < nsegs)
                copy_seg_run(srun, P.run + pf);
            cp_async_wait_all();
            misc[0] = pf;
        }
        __syncthreads();
        const int item = misc[0];
        if (item >= nsegs)
            break;
        const SegRun d = *srun;
        if (tid == 0) {
            pf = i0 + atomicAdd(&P.cnt->work_seg, 1);  // consumed after the staging
            pf_copied = false;
        }
        const int row = d.row;
        const int a0 = d.a0;
        const int k = d.k;
        const int span = d.c_hi - d.c_lo;
        // distinct columns of the row up to the next segment (checked at the end)
        const int next_u = d.next_u;
        const int nsum = (span + 1023) >> 10;
        const int *sp0 = P.split + d.sp;
        const int *sp1 = sp0 + k;
        // nonempty sub-lists of the segment, in leaf order (a thread takes
        // four consecutive lists per pass: hub rows have thousands of lists
        // and few products of each in one segment)
        constexpr int LPT = 4;
        int lcarry = 0, pcarry = 0;
        for (int lb = 0; lb < k; lb += NT * LPT) {
            int st[LPT], len[LPT];
            int cnt = 0, psum = 0;
#pragma unroll
            for (int q = 0; q < LPT; q++) {
                const int l = lb + tid * LPT + q;
                st[q] = 0;
                len[q] = 0;
                if (l < k) {
                    st[q] = sp0[l];
                    len[q] = sp1[l] - st[q];
                }
                cnt += len[q] > 0;
                psum += len[q];
            }
            long long tot;
            const long long ex = block_excl_scan<NT, long long>(
                ((long long)cnt << 32) | (long long)psum, ws, &tot);
            int li = lcarry + (int)(ex >> 32);
            int po = pcarry + (int)(ex & 0xffffffffLL);
#pragma unroll
            for (int q = 0; q < LPT; q++) {
                if (len[q] > 0) {
                    if (li < kSegCap) {
                        loff[li] = po;
                        lbs[li] = st[q];
                        lleaf[li] = (unsigned short)(lb + tid * LPT + q);
                    }
                    li++;
                    po += len[q];
                }
            }
            lcarry += (int)(tot >> 32);
            pcarry += (int)(tot & 0xffffffffLL);
        }
        const int nlists = lcarry, nprod = pcarry;
        if (nprod > kSegCap || nprod != d.nprod || nsum > kSumWords || span <= 0) {
            if (tid == 0)
                atomicOr(&P.cnt->err, kErrWindowOverflow);
            continue;
        }
        if (tid == 0) {
            loff[nlists] = nprod;
            misc[1] = 0;  // long runs
            misc[2] = 0;  // staged column out of range
            misc[3] = 0;  // listed columns of three or four products
            misc[4] = 0;  // listed columns of five to eight products
        }
        // a segment spanning at most 32 * kSegCap columns ranks its columns
        // with one flat bitmap in cw (a prefix per word); wider ones with a
        // summary bit per nonempty word and compressed words
        const bool flat = span <= 32 * kSegCap;
        const int nwf = (span + 31) >> 5;
        if (flat) {
            for (int i = tid; i < nwf; i += NT)
                cw[i] = 0;
        } else {
            for (int i = tid; i < nsum; i += NT)
                summ[i] = 0;
        }
        __syncthreads();
        // stage products in list-major (= leaf) order; mark their words in the
        // flat bitmap or in the summary
        const int ipt = (nprod + NT - 1) / NT;
        const int p0 = min(tid * ipt, nprod), p1 = min(p0 + ipt, nprod);
        // a thread's products are column-sorted within each list, so runs of
        // equal summary words are OR-ed in a register and flushed once
        unsigned run_w = 0xffffffffu, run_b = 0;
        if (p0 < p1) {
            int j = last_le(loff, nlists, p0);
            int lbeg = loff[j], lend = loff[j + 1], bsj = lbs[j];
            for (int p = p0; p < p1; p += kGatherBatch) {
                const int n = min(kGatherBatch, p1 - p);
                int addr[kGatherBatch], lid[kGatherBatch], c[kGatherBatch];
                T bv[kGatherBatch], av[kGatherBatch];
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++) {
                    if (i < n) {
                        while (p + i >= lend) {
                            j++;
                            lbeg = lend;
                            lend = loff[j + 1];
                            bsj = lbs[j];
                        }
                        addr[i] = bsj + (p + i - lbeg);
                        lid[i] = j;
                    }
                }
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++) {
                    if (i < n) {
                        const bool in = BRM_IN(P.cnt, addr[i], B.nnz);
                        c[i] = in ? bcol[addr[i]] : d.c_lo;
                        bv[i] = in ? bval[addr[i]] : T(0);
                        av[i] = aval[a0 + lleaf[lid[i]]];
                    }
                }
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++) {
                    if (i < n) {
                        const int e = p + i;
                        int rc = c[i] - d.c_lo;
                        if ((unsigned)rc >= (unsigned)span) {
                            misc[2] = 1;
                            rc = 0;
                        }
                        prc[e] = rc;
                        pval[e] = vmul(av[i], bv[i]);
                        pleaf[e] = lleaf[lid[i]];
                        const unsigned sw = (unsigned)rc >> (flat ? 5 : 10);
                        if (sw != run_w) {
                            if (run_b)
                                atomicOr(flat ? &cw[run_w] : &summ[run_w], run_b);
                            run_w = sw;
                            run_b = 0;
                        }
                        run_b |= 1u << ((rc >> (flat ? 0 : 5)) & 31);
                    }
                }
            }
            if (run_b)
                atomicOr(flat ? &cw[run_w] : &summ[run_w], run_b);
        }
        __syncthreads();
        // every thread has read this segment's record: copy the next one
        if (tid == 0 && pf < nsegs) {
            copy_seg_run(srun, P.run + pf);
            pf_copied = true;
        }
        if (misc[2]) {  // a column outside the segment: the plan does not match the input
            if (tid == 0)
                atomicOr(&P.cnt->err, kErrBadInput);
            continue;
        }
        // compressed words: one per nonempty 32-column word (flat: every word)
        int ncw = nwf;
        if (!flat) {
            // SPT consecutive summary words a thread (nsum <= kSumWords)
            constexpr int SPT = (kSumWords + NT - 1) / NT;
            const int s0 = min(tid * SPT, nsum), s1 = min(s0 + SPT, nsum);
            int sc = 0;
            for (int i = s0; i < s1; i++)
                sc += __popc(summ[i]);
            long long ncw_t;
            int sx = (int)block_excl_scan<NT, long long>(sc, ws, &ncw_t);
            for (int i = s0; i < s1; i++) {
                srank[i] = (unsigned short)sx;
                sx += __popc(summ[i]);
            }
            ncw = (int)ncw_t;
            for (int i = tid; i < ncw; i += NT)
                cw[i] = 0;
            for (int i = tid; i <= nprod; i += NT)  // the sub-list table is dead now
                ucnt[i] = 0;
            __syncthreads();
        }
        // mark the compressed words; keep each product's word index in pu
        if (!flat) {
            int run_ci = -1;
            unsigned bits = 0;
            for (int p = p0; p < p1; p++) {
                const int rc = prc[p];
                const int w = rc >> 5;
                const int ci = srank[w >> 5] + __popc(summ[w >> 5] & ((1u << (w & 31)) - 1u));
                pu[p] = (unsigned short)ci;
                if (ci != run_ci) {
                    if (bits)
                        atomicOr(&cw[run_ci], bits);
                    run_ci = ci;
                    bits = 0;
                }
                bits |= 1u << (rc & 31);
            }
            if (bits)
                atomicOr(&cw[run_ci], bits);
            __syncthreads();
        } else {
            // a flat segment clears the column counts here (the sub-list
            // table they overwrite is dead since the staging barrier); the
            // barrier of the rank scan below orders them before the counting
            for (int i = tid; i <= nprod; i += NT)
                ucnt[i] = 0;
        }
        // ranks of the compressed words -> distinct columns before each word
        long long U_t;
        {
            const int cpt = (ncw + NT - 1) / NT;
            const int c0 = min(tid * cpt, ncw), c1 = min(c0 + cpt, ncw);
            int cs = 0;
            for (int i = c0; i < c1; i++)
                cs += __popc(cw[i]);
            int r = (int)block_excl_scan<NT, long long>(cs, ws, &U_t);
            for (int i = c0; i < c1; i++) {
                cwr[i] = (unsigned short)r;
                r += __popc(cw[i]);
            }
        }
        const int U = (int)U_t;
        const bool nodup = (U == nprod);
        __syncthreads();
        // u = distinct-column rank of each product; count the products of
        // every column (the rank within a column, from the atomic, is in
        // arbitrary order and is put in leaf order when the column is reduced)
        for (int p = p0; p < p1; p++) {
            const int rc = prc[p];
            const int ci = flat ? rc >> 5 : pu[p];
            const int u = cwr[ci] + __popc(cw[ci] & ((1u << (rc & 31)) - 1u));
            pu[p] = (unsigned short)u;
            if (!nodup && BRM_IN(P.cnt, u, U))
                ia[p] = (unsigned short)atomicAdd(&ucnt[u], 1);
        }
        __syncthreads();
        const long long obase = (UPPER ? P.scan_flop[row] : (long long)crpt[row]) + d.u_off;
        unsigned short *S = ib;
        if (nodup) {
            // every column has one contribution: position u holds product e
            for (int p = p0; p < p1; p++)
                if (BRM_IN(P.cnt, pu[p], nprod))
                    S[pu[p]] = (unsigned short)p;
        } else {
            // exclusive scan of the column counts (in place), then scatter
            const int cpt = (U + NT - 1) / NT;
            const int c0 = min(tid * cpt, U), c1 = min(c0 + cpt, U);
            int cs = 0;
            for (int i = c0; i < c1; i++)
                cs += ucnt[i];
            long long tot;
            int r = (int)block_excl_scan<NT, long long>(cs, ws, &tot);
            for (int i = c0; i < c1; i++) {
                const int c = ucnt[i];
                ucnt[i] = r;
                r += c;
            }
            if (tid == 0)
                ucnt[U] = nprod;
            __syncthreads();
            for (int p = p0; p < p1; p++)
                if (BRM_IN(P.cnt, ucnt[pu[p]] + ia[p], nprod))
                    S[ucnt[pu[p]] + ia[p]] = (unsigned short)p;
        }
        __syncthreads();
        // one thread per output column of one or two products (consecutive
        // columns -> coalesced stores); columns of three or four and of five to
        // eight products are listed (at the front and the back of pu, dead
        // after the scatter) and reduced by a second, dense pass, so that the
        // lanes of a warp run the same code; longer columns go to longu
        for (int u = tid; u < U; u += NT) {
            int i0 = u, len = 1;
            if (!nodup) {
                i0 = ucnt[u];
                len = ucnt[u + 1] - i0;
            }
            const int e0 = S[i0];
            T v;
            if (len == 1) {
                v = pval[e0];
            } else if (len == 2) {
                const int e1 = S[i0 + 1];
                v = pleaf[e0] < pleaf[e1] ? vadd(pval[e0], pval[e1])   // left + right
                                          : vadd(pval[e1], pval[e0]);
            } else if (len <= 4) {
                pu[atomicAdd(&misc[3], 1)] = (unsigned short)u;
                continue;
            } else if (len <= 8) {
                pu[kSegCap - 1 - atomicAdd(&misc[4], 1)] = (unsigned short)u;
                continue;
            } else {
                const int li = atomicAdd(&misc[1], 1);
                if (li < kLongMax)
                    longu[li] = (unsigned short)u;
                continue;
            }
            if (BRM_IN(P.cnt, obase + u, P.c_cap)) {
                ccol[obase + u] = d.c_lo + prc[e0];
                cval[obase + u] = v;
            }
        }
        __syncthreads();
        const int n34 = misc[3], nmid = n34 + misc[4];
        for (int i = tid; i < nmid; i += NT) {
            const int u = i < n34 ? pu[i] : pu[kSegCap - 1 - (i - n34)];
            const int i0 = ucnt[u], len = ucnt[u + 1] - i0;
            const int e0 = S[i0];
            T v;
            if (len <= 4) {
                // sort the (leaf, value) pairs in registers, then the closed form
                const int e1 = S[i0 + 1], e2 = S[i0 + 2];
                int l0 = pleaf[e0], l1 = pleaf[e1], l2 = pleaf[e2];
                T v0 = pval[e0], v1 = pval[e1], v2 = pval[e2];
                if (len == 3) {
                    leaf_cas(l0, v0, l1, v1);
                    leaf_cas(l1, v1, l2, v2);
                    leaf_cas(l0, v0, l1, v1);
                    v = trie3(l0, l1, l2, v0, v1, v2);
                } else {
                    const int e3 = S[i0 + 3];
                    int l3 = pleaf[e3];
                    T v3 = pval[e3];
                    leaf_cas(l0, v0, l1, v1);
                    leaf_cas(l2, v2, l3, v3);
                    leaf_cas(l0, v0, l2, v2);
                    leaf_cas(l1, v1, l3, v3);
                    leaf_cas(l1, v1, l2, v2);
                    v = trie4(l0, l1, l2, l3, v0, v1, v2, v3);
                }
            } else {
                // sorting network and a register stack
                int l8[8];
                T v8[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    if (j < len) {
                        const int e = S[i0 + j];
                        l8[j] = pleaf[e];
                        v8[j] = pval[e];
                    } else {
                        l8[j] = INT_MAX;
                        v8[j] = T(0);
                    }
                }
                leaf_sort8(l8, v8);
                RegShiftReduce<T, 8> sr;
                sr.init(l8[0], v8[0]);
#pragma unroll
                for (int j = 1; j < 8; j++)
                    if (j < len)
                        sr.push(l8[j], v8[j]);
                v = sr.finish();
            }
            if (BRM_IN(P.cnt, obase + u, P.c_cap)) {
                ccol[obase + u] = d.c_lo + prc[e0];
                cval[obase + u] = v;
            }
        }
        __syncthreads();
        // columns with more than eight products: one warp each puts them in
        // leaf order (= staging order p, which it ranks with a bitmap over
        // p) and hands them to the column reducer through the long-column
        // scratch; when the scratch is full it reduces them itself (across
        // its lanes up to 32 products, in its first lane beyond)
        const int nlong = min(misc[1], kLongMax);
        {
            const int lane = tid & 31, wid = tid >> 5;
            unsigned *bmp = cw + wid * kSegPWords;
            unsigned short *wpre = (unsigned short *)(cw + L::NW * kSegPWords) + wid * kSegPWords;
            const int nwp = (nprod + 31) >> 5;
            T *lval = (T *)P.long_val;
            for (int lb = wid; lb < nlong; lb += 32 * L::NW) {
              // the warp's next (up to) 32 columns lb + j * NW: one
              // reservation of long-column scratch covers all of them
              const int lj = lb + lane * L::NW;
              int myu = 0, mylen = 0;
              if (lj < nlong) {
                  myu = longu[lj];
                  mylen = ucnt[myu + 1] - ucnt[myu];
              }
              const int ncol = __popc(__ballot_sync(kFull, lj < nlong));
              const int lincl = warp_incl_scan(mylen);
              unsigned long long rcol = 0, relem = 0;
              if (lane == 31) {
                  rcol = atomicAdd(&P.cnt->long_cols, (unsigned long long)ncol);
                  relem = atomicAdd(&P.cnt->long_elems, (unsigned long long)lincl);
              }
              rcol = __shfl_sync(kFull, rcol, 31);
              relem = __shfl_sync(kFull, relem, 31);
              for (int jc = 0; jc < ncol; jc++) {
                const int u = __shfl_sync(kFull, myu, jc);
                const int len = __shfl_sync(kFull, mylen, jc);
                const int i0 = ucnt[u], i1 = i0 + len;
                const long long lci = (long long)rcol + jc;
                const long long leo = (long long)relem + __shfl_sync(kFull, lincl - mylen, jc);
                const bool handoff = lci < P.long_cap_cols && leo + len <= P.long_cap_elems;
                for (int w = lane; w < nwp; w += 32)
                    bmp[w] = 0;
                __syncwarp();
                for (int i = i0 + lane; i < i1; i += 32) {
                    const int p = S[i];
                    atomicOr(&bmp[p >> 5], 1u << (p & 31));
                }
                __syncwarp();
                {
                    const int w0 = lane * 3;
                    const int c0 = w0 < nwp ? __popc(bmp[w0]) : 0;
                    const int c1 = w0 + 1 < nwp ? __popc(bmp[w0 + 1]) : 0;
                    const int c2 = w0 + 2 < nwp ? __popc(bmp[w0 + 2]) : 0;
                    const int ex = warp_incl_scan(c0 + c1 + c2) - (c0 + c1 + c2);
                    if (w0 < nwp)
                        wpre[w0] = (unsigned short)ex;
                    if (w0 + 1 < nwp)
                        wpre[w0 + 1] = (unsigned short)(ex + c0);
                    if (w0 + 2 < nwp)
                        wpre[w0 + 2] = (unsigned short)(ex + c0 + c1);
                }
                __syncwarp();
                for (int i = i0 + lane; i < i1; i += 32) {
                    const int p = S[i];
                    const int r = wpre[p >> 5] + __popc(bmp[p >> 5] & ((1u << (p & 31)) - 1u));
                    if (handoff) {
                        P.long_leaf[leo + r] = pleaf[p];
                        lval[leo + r] = pval[p];
                    } else {
                        if (BRM_IN(P.cnt, i0 + r, nprod))
                            ia[i0 + r] = (unsigned short)p;
                    }
                }
                if (lci < P.long_cap_cols && lane == 0) {
                    LongCol c;
                    c.out = obase + u;
                    c.off = leo;
                    c.col = d.c_lo + prc[S[i0]];
                    c.len = handoff ? len : -1;
                    P.long_col[lci] = c;
                }
                __syncwarp();
                if (handoff)
                    continue;
                if (len <= 32) {
                    const int e = ia[i0 + (lane < len ? lane : 0)];
                    const T r = warp_trie<T>(pleaf[e], pval[e], len);
                    if (lane == 0) {
                        if (BRM_IN(P.cnt, obase + u, P.c_cap)) {
                            ccol[obase + u] = d.c_lo + prc[e];
                            cval[obase + u] = r;
                        }
                    }
                } else if (lane == 0) {
                    ShiftReduce<T, 17> sr;
                    sr.init(pleaf[ia[i0]], pval[ia[i0]]);
                    for (int i = i0 + 1; i < i1; i++)
                        sr.push(pleaf[ia[i]], pval[ia[i]]);
                    if (BRM_IN(P.cnt, obase + u, P.c_cap)) {
                        ccol[obase + u] = d.c_lo + prc[ia[i0]];
                        cval[obase + u] = sr.finish();
                    }
                }
                __syncwarp();
              }
            }
        }
        // the segment must produce exactly its share of the row's columns
        if (tid == 0 && U != next_u - d.u_off)
            atomicOr(&P.cnt->err, kErrNnzMismatch);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// 4. column reducer: one thread per long column handed over by the segment
//    kernel; its products are in leaf order, so the trie is one ShiftReduce
//    pass with the stack in registers (leaves below 2^16: at most 16 entries
//    below the top).
// ---------------------------------------------------------------------------
// Sequential trie of the elements [b, e) of a long column (leaves in
// increasing order, below 2^(D-1)); the elements are loaded GB at a time, so
// a long column does not wait for one load per element.
template <typename T, int D, int GB = kGatherBatch>
__device__ __forceinline__ T long_run(const unsigned short *__restrict__ lleaf,
                                      const T *__restrict__ lval, long long b, long long e)
{
    RegShiftReduce<T, D> sr;
    sr.init(lleaf[b], lval[b]);
    for (long long j0 = b + 1; j0 < e; j0 += GB) {
        int lf[GB];
        T lv[GB];
#pragma unroll
        for (int q = 0; q < GB; q++) {
            if (j0 + q < e) {
                lf[q] = lleaf[j0 + q];
                lv[q] = lval[j0 + q];
            }
        }
#pragma unroll
        for (int q = 0; q < GB; q++)
            if (j0 + q < e)
                sr.push(lf[q], lv[q]);
    }
    return sr.finish();
}

constexpr int kLrWarpMin = 32;  // columns with more products are reduced by a whole warp
                                // (and so are columns with leaves of 4096 or more)

// A long column reduced by a whole warp.  Its leaves (strictly increasing,
// below 2^bits) are cut into the 32 aligned ranges of 2^s leaves, s = bits - 5:
// every range is one subtree of the merge tree at level s, so lane j reduces
// the products of range j on its own (at most s split levels: 12 stack
// entries suffice for 16-bit leaves), and the subtree values are then joined
// by the trie over their range indices (warp_trie); every lane returns the
// value.  cnt and sv are the warp's 32-entry shared scratch.
template <typename T>
__device__ __forceinline__ T warp_long_column(const unsigned short *__restrict__ lleaf,
                                              const T *__restrict__ lval, long long b, int len,
                                              int *cnt, T *sv)
{
    const int lane = threadIdx.x & 31;
    const int bits = 32 - __clz((int)lleaf[b + len - 1] | 1);
    const int s = bits > 5 ? bits - 5 : 0;
    cnt[lane] = 0;
    __syncwarp();
    for (int p = lane; p < len; p += 32)
        atomicAdd(&cnt[lleaf[b + p] >> s], 1);
    __syncwarp();
    const int mc = cnt[lane];
    const int lo = warp_incl_scan(mc) - mc;
    T v = T(0);
    if (mc > 0)
        v = long_run<T, 12, 4>(lleaf, lval, b + lo, b + lo + mc);
    // the nonempty ranges in order, one per lane
    const unsigned hm = __ballot_sync(kFull, mc > 0);
    const int r = __popc(hm & ((1u << lane) - 1u));
    __syncwarp();
    if (mc > 0) {
        sv[r] = v;
        cnt[r] = lane;
    }
    __syncwarp();
    const int nh = __popc(hm);
    const int li = lane < nh ? cnt[lane] : 0;
    const T vi = lane < nh ? sv[lane] : T(0);
    __syncwarp();
    return __shfl_sync(kFull, warp_trie<T>(li, vi, nh), 0);  // the trie's value is in lane 0
}

// Columns of at most kLrWarpMin products with leaves below 4096 are reduced
// one per thread (k_long_reduce), the others by whole warps (k_long_warp):
// two kernels, so that neither pays the other's registers.
__device__ __forceinline__ bool long_by_thread(const LongCol &c, int last)
{
    return c.len <= kLrWarpMin && last < 4096;
}

template <typename T>
__global__ void __launch_bounds__(128) k_long_reduce(PlanDev P, int *ccol, T *cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    const long long n = min((long long)P.cnt->long_cols, P.long_cap_cols);
    const T *__restrict__ lval = (const T *)P.long_val;
    const unsigned short *__restrict__ lleaf = P.long_leaf;
    for (long long i0 = (long long)blockIdx.x * blockDim.x; i0 < n;
         i0 += (long long)gridDim.x * blockDim.x) {
        const long long i = i0 + threadIdx.x;
        LongCol c;
        c.len = 0;
        if (i < n)
            c = P.long_col[i];
        if (c.len > 0 && !BRM_IN(P.cnt, c.off + c.len - 1, P.long_cap_elems))
            c.len = 0;  // checked build: a record outside the scratch is skipped
        const int last = c.len > 0 ? (int)lleaf[c.off + c.len - 1] : 0;
        const bool mine = c.len > 0 && long_by_thread(c, last);
        // the stack depth follows the warp's largest last leaf
        const int top = __reduce_max_sync(kFull, mine ? last : 0);
        if (mine) {
            if (BRM_IN(P.cnt, c.out, P.c_cap) &&
                BRM_IN(P.cnt, c.off + c.len - 1, P.long_cap_elems)) {
                ccol[c.out] = c.col;
                cval[c.out] = top < 256 ? long_run<T, 9>(lleaf, lval, c.off, c.off + c.len)
                                    : long_run<T, 13, 4>(lleaf, lval, c.off, c.off + c.len);
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(128) k_long_warp(PlanDev P, int *ccol, T *cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    __shared__ int s_cnt[4][32];
    __shared__ T s_val[4][32];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long n = min((long long)P.cnt->long_cols, P.long_cap_cols);
    const T *__restrict__ lval = (const T *)P.long_val;
    const unsigned short *__restrict__ lleaf = P.long_leaf;
    for (long long i0 = (long long)blockIdx.x * blockDim.x; i0 < n;
         i0 += (long long)gridDim.x * blockDim.x) {
        const long long i = i0 + threadIdx.x;
        LongCol c;
        c.len = 0;
        if (i < n)
            c = P.long_col[i];
        if (c.len > 0 && !BRM_IN(P.cnt, c.off + c.len - 1, P.long_cap_elems))
            c.len = 0;  // checked build: a record outside the scratch is skipped
        const int last = c.len > 0 ? (int)lleaf[c.off + c.len - 1] : 0;
        unsigned lm = __ballot_sync(kFull, c.len > 0 && !long_by_thread(c, last));
        while (lm) {
            const int src = __ffs(lm) - 1;
            lm &= lm - 1u;
            const long long off = __shfl_sync(kFull, c.off, src);
            const int len = __shfl_sync(kFull, c.len, src);
            const T r = warp_long_column<T>(lleaf, lval, off, len, s_cnt[wid], s_val[wid]);
            if (lane == src) {
                if (BRM_IN(P.cnt, c.out, P.c_cap) &&
                    BRM_IN(P.cnt, c.off + c.len - 1, P.long_cap_elems)) {
                    ccol[c.out] = c.col;
                    cval[c.out] = r;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// 5. segments grouped by row parts: for a numeric phase run part by part
//    (rows [pb[p], pb[p+1]) for p < nparts), the segment list is reordered so
//    every part's segments are contiguous, and ranges[2p], ranges[2p+1] give
//    the part's slice.  cnt (nparts ints) must be zero before the count pass.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int part_of_row(const int *pb, int nparts, int row)
{
    int p = 0;
    while (p + 1 < nparts && row >= pb[p + 1])
        p++;
    return p;
}

template <int UNUSED = 0>
__global__ void __launch_bounds__(256) k_seg_part_count(PlanDev P, const int *pb, int nparts,
                                                        int *cnt)
{
    const int n = P.cnt->n_seg;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&cnt[part_of_row(pb, nparts, P.seg[P.seg_list[i]].row)], 1);
}

template <int UNUSED = 0>
__global__ void __launch_bounds__(256) k_seg_part_scatter(PlanDev P, const int *pb, int nparts,
                                                          const int *cnt, int *fill, int *out,
                                                          int *ranges)
{
    __shared__ int base[kMaxParts + 1];
    if (threadIdx.x == 0) {
        int s = 0;
        for (int p = 0; p < nparts; p++) {
            base[p] = s;
            s += cnt[p];
        }
        base[nparts] = s;
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x < nparts) {
        ranges[2 * threadIdx.x] = base[threadIdx.x];
        ranges[2 * threadIdx.x + 1] = base[threadIdx.x + 1];
    }
    const int n = P.cnt->n_seg;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int slot = P.seg_list[i];
        const int p = part_of_row(pb, nparts, P.seg[slot].row);
        out[base[p] + atomicAdd(&fill[p], 1)] = slot;
    }
}

}  // namespace brm
