// brm_seg.cuh -- segmented processing of heavy rows.
//
// A heavy row (more products or lists than a mid-row batch holds) is cut into
// column segments [c_lo, c_hi).  Columns of C are independent, so the merge
// tree of the row restricted to a column range is the same tree with every
// list restricted to that range (BRMerge-SpGEMM/inc/spgemm.h:639-707): the
// leaf index of a product, and therefore the order of its additions, does
// not depend on the cut.  Three steps:
//
//   1. planning (symbolic phase, one CTA per heavy row): a bitmap of the
//      row's columns and a product count per 32-column word over chunks of
//      kPlanBits columns give the row's exact nnz and the cut points: a cut
//      before word w when the running product count crosses a multiple of
//      kSegCut, around words holding more than kSegCut products, and every
//      kSegSpan columns; each segment then holds <= kSegCap products.  The
//      segment's output offset within the row (distinct columns before c_lo)
//      comes from the same bitmap.
//   2. split table (numeric phase): for every segment boundary and every list
//      of the row, the first list position at or after the boundary column
//      (one independent binary search per entry).
//   3. segment kernel (numeric phase, one CTA pass per segment): stage the
//      segment's products in list-major order, stable LSD radix sort on the
//      column offset c - c_lo (< 2^kSegSpanBits, two 8-bit passes), then one
//      thread per output column evaluates the merge tree with ShiftReduce.
#pragma once

#include <climits>

#include "brm_common.cuh"
#include "brm_mid.cuh"
#include "brm_plan.h"

namespace brm {

constexpr int kPlanThreads = 512;

constexpr int kDenseMax = 128;  // dense words per planning chunk with per-column counts

struct PlanLayout {
    static constexpr size_t o_bm = 0;
    static constexpr size_t o_hist = o_bm + kPlanWords * 4;
    static constexpr size_t o_dix = o_hist + kPlanWords * 4;
    static constexpr size_t o_ccnt = o_dix + kPlanWords * 2;
    static constexpr size_t o_ws = o_ccnt + kDenseMax * 32 * 4;
    static constexpr size_t o_misc = o_ws + (kPlanThreads / 32 + 1) * 8;
    static constexpr size_t bytes = o_misc + 64;
};

// Walks the segment starts of planning word w (chunk-relative) in column
// order and calls f(column_in_word, product_prefix, distinct_prefix) for
// each.  `run` packs (products << 32 | distinct columns) before word w and
// ph is the product count of word w-1.  A word with more than kSegCut
// products is always cut before and after; inside it, a new segment starts
// at a column when the running product count would exceed kSegCut.
template <typename Fn>
__device__ __forceinline__ void plan_word_starts(int w, unsigned h, unsigned ph,
                                                 unsigned long long run, unsigned bits,
                                                 const unsigned *ccnt, Fn f)
{
    const unsigned pe = (unsigned)(run >> 32);
    const unsigned ue = (unsigned)(run & 0xffffffffu);
    if (h > (unsigned)kSegCut) {
        f(0, pe, ue);
        unsigned acc = 0, pp = pe;
        for (int c = 0; c < 32; c++) {
            const unsigned cc = ccnt[c];
            if (cc == 0)
                continue;
            if (acc > 0 && acc + cc > (unsigned)kSegCut) {
                f(c, pp, ue + __popc(bits & ((1u << c) - 1u)));
                acc = 0;
            }
            acc += cc;
            pp += cc;
        }
        return;
    }
    const bool start = (w == 0) || ph > (unsigned)kSegCut || (pe / kSegCut) != ((pe - ph) / kSegCut) ||
                       ((w & (kSegSpan / 32 - 1)) == 0);
    if (start)
        f(0, pe, ue);
}

// ---------------------------------------------------------------------------
// 1. planning
// ---------------------------------------------------------------------------
template <int UNUSED = 0>
__global__ void __launch_bounds__(kPlanThreads) k_heavy_plan(CsrDev A, CsrDev B, PlanDev P)
{
    constexpr int NT = kPlanThreads;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned *bm = (unsigned *)(smem + PlanLayout::o_bm);
    unsigned *hist = (unsigned *)(smem + PlanLayout::o_hist);
    unsigned short *dix = (unsigned short *)(smem + PlanLayout::o_dix);
    unsigned *ccnt = (unsigned *)(smem + PlanLayout::o_ccnt);
    long long *ws = (long long *)(smem + PlanLayout::o_ws);
    int *misc = (int *)(smem + PlanLayout::o_misc);
    const int tid = threadIdx.x;
    const int M = A.M;
    const int nrows = P.cnt->bin_count[kBinHeavy];
    const int *rows = P.rows + (size_t)kBinHeavy * M;
    const int *__restrict__ bcol = B.col;
    for (;;) {
        if (tid == 0)
            misc[0] = atomicAdd(&P.cnt->work_plan, 1);
        __syncthreads();
        const int item = misc[0];
        __syncthreads();
        if (item >= nrows)
            break;
        const int row = rows[item];
        const int a0 = A.rpt[row];
        const int k = A.rpt[row + 1] - a0;
        const long long F = P.flop[row];
        const unsigned long long base = P.seg_base[row];
        const unsigned long long bound = seg_bound(F, B.N);
        int mn = INT_MAX, mx = -1;
        for (int l = tid; l < k; l += NT) {
            const int len = P.alen[a0 + l];
            if (len > 0) {
                const int s = P.abs[a0 + l];
                mn = min(mn, bcol[s]);
                mx = max(mx, bcol[s + len - 1]);
            }
        }
        mn = (int)block_min<NT, long long>(mn, ws);
        mx = (int)block_max<NT, long long>(mx, ws);
        if (mx < 0 || mn < 0 || mx >= B.N) {
            if (tid == 0) {
                if (mx >= 0)
                    atomicOr(&P.cnt->err, kErrBadInput);
                P.nnz[row] = 0;
                P.seg_n[row] = 0;
            }
            continue;
        }
        // lanes per list: about avg / kGatherBatch, a power of two in [1, 32]
        const int G = group_size(F / kGatherBatch, k);
        const int lg = tid & (G - 1);
        long long u_run = 0;
        int nseg = 0;
        bool fail = false;
        for (long long clo = mn; clo <= mx; clo += kPlanBits) {
            const int lo = (int)clo;
            const int chi = (int)min((long long)mx + 1, clo + kPlanBits);
            const int span = chi - lo;
            const int nw = (span + 31) >> 5;
            const bool multi = (long long)mx + 1 - mn > kPlanBits;
            for (int i = tid; i < nw; i += NT) {
                bm[i] = 0;
                hist[i] = 0;
            }
            __syncthreads();
            // pass over the chunk's products: column bitmap and products per word
            for (int l = tid / G; l < k; l += NT / G) {
                const int len = P.alen[a0 + l];
                if (len == 0)
                    continue;
                int s = P.abs[a0 + l], e = s + len;
                if (multi) {
                    s = lower_bound_idx(bcol, s, e, lo);
                    e = lower_bound_idx(bcol, s, e, chi);
                }
                for (int idx = s + lg; idx < e; idx += G * kGatherBatch) {
                    int c[kGatherBatch];
#pragma unroll
                    for (int i = 0; i < kGatherBatch; i++)
                        c[i] = (idx + i * G < e) ? bcol[idx + i * G] : -1;
#pragma unroll
                    for (int i = 0; i < kGatherBatch; i++) {
                        if (idx + i * G < e) {
                            const int rc = c[i] - lo;
                            if ((unsigned)rc < (unsigned)span) {
                                atomicOr(&bm[rc >> 5], 1u << (rc & 31));
                                atomicAdd(&hist[rc >> 5], 1u);
                            } else {
                                atomicOr(&P.cnt->err, kErrBadInput);
                            }
                        }
                    }
                }
            }
            __syncthreads();
            const int wpt = (nw + NT - 1) / NT;
            const int w0 = min(tid * wpt, nw), w1 = min(w0 + wpt, nw);
            // dense words get per-column product counts (second pass)
            int nd_local = 0;
            unsigned long long sp = 0;
            for (int w = w0; w < w1; w++) {
                const unsigned h = hist[w];
                nd_local += h > (unsigned)kSegCut ? 1 : 0;
                sp += ((unsigned long long)h << 32) | (unsigned)__popc(bm[w]);
            }
            long long ndt;
            int dx = (int)block_excl_scan<NT, long long>(nd_local, ws, &ndt);
            const int nd = (int)ndt;
            if (nd > kDenseMax)
                fail = true;  // uniform
            if (!fail && nd > 0) {
                for (int w = w0; w < w1; w++)
                    if (hist[w] > (unsigned)kSegCut)
                        dix[w] = (unsigned short)dx++;
                for (int i = tid; i < nd * 32; i += NT)
                    ccnt[i] = 0;
                __syncthreads();
                for (int l = tid / G; l < k; l += NT / G) {
                    const int len = P.alen[a0 + l];
                    if (len == 0)
                        continue;
                    int s = P.abs[a0 + l], e = s + len;
                    if (multi) {
                        s = lower_bound_idx(bcol, s, e, lo);
                        e = lower_bound_idx(bcol, s, e, chi);
                    }
                    for (int idx = s + lg; idx < e; idx += G * kGatherBatch) {
                        int c[kGatherBatch];
#pragma unroll
                        for (int i = 0; i < kGatherBatch; i++)
                            c[i] = (idx + i * G < e) ? bcol[idx + i * G] : -1;
#pragma unroll
                        for (int i = 0; i < kGatherBatch; i++) {
                            if (idx + i * G < e) {
                                const int rc = c[i] - lo;
                                if ((unsigned)rc < (unsigned)span && hist[rc >> 5] > (unsigned)kSegCut)
                                    atomicAdd(&ccnt[dix[rc >> 5] * 32 + (rc & 31)], 1u);
                            }
                        }
                    }
                }
                __syncthreads();
                bool big = false;
                for (int i = tid; i < nd * 32; i += NT)
                    big |= ccnt[i] > (unsigned)kSegCap;
                fail = __syncthreads_or(big) != 0;
            }
            long long tot;
            const unsigned long long ex = (unsigned long long)block_excl_scan<NT, long long>(
                (long long)sp, ws, &tot);
            // count the chunk's segment starts
            int nstart = 0;
            if (!fail) {
                unsigned long long run = ex;
                unsigned ph = (w0 > 0 && w0 < nw) ? hist[w0 - 1] : 0u;
                for (int w = w0; w < w1; w++) {
                    const unsigned h = hist[w];
                    plan_word_starts(w, h, ph, run, bm[w],
                                     h > (unsigned)kSegCut ? ccnt + dix[w] * 32 : ccnt,
                                     [&](int, unsigned, unsigned) { nstart++; });
                    run += ((unsigned long long)h << 32) | (unsigned)__popc(bm[w]);
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
                continue;  // keep counting distinct columns; the row takes the spill path
            }
            // write the chunk's segments: c_lo, u_off and the product prefix
            {
                unsigned long long run = ex;
                unsigned ph = (w0 > 0 && w0 < nw) ? hist[w0 - 1] : 0u;
                int r = sx;
                for (int w = w0; w < w1; w++) {
                    const unsigned h = hist[w];
                    plan_word_starts(w, h, ph, run, bm[w],
                                     h > (unsigned)kSegCut ? ccnt + dix[w] * 32 : ccnt,
                                     [&](int c, unsigned pe, unsigned ue) {
                                         SegDesc &d = P.seg[base + nseg + r];
                                         d.row = row;
                                         d.c_lo = lo + 32 * w + c;
                                         d.u_off = (int)(u_chunk + (long long)ue);
                                         d.bidx = nseg + r;
                                         d.nprod = (int)pe;  // prefix; a count below
                                         r++;
                                     });
                    run += ((unsigned long long)h << 32) | (unsigned)__popc(bm[w]);
                    ph = h;
                }
            }
            __syncthreads();  // descriptors of this chunk visible to the block
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
                P.seg[base + i].tab = tab;
                P.seg_list[lpos + i] = (int)(base + i);
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
    const int nsegs = P.cnt->n_seg;
    const int *__restrict__ bcol = B.col;
    for (int it = blockIdx.x; it < nsegs; it += gridDim.x) {
        const int slot = P.seg_list[it];
        const int row = P.seg[slot].row;
        const int b = P.seg[slot].bidx;
        const int c_lo = P.seg[slot].c_lo;
        const long long tab = P.seg[slot].tab;
        const int nseg = P.seg_n[row];
        const int a0 = A.rpt[row];
        const int k = A.rpt[row + 1] - a0;
        int *t0 = P.split + tab + (long long)b * k;
        for (int l = threadIdx.x; l < k; l += blockDim.x) {
            const int s = P.abs[a0 + l];
            const int e = s + P.alen[a0 + l];
            t0[l] = (b == 0) ? s : lower_bound_idx(bcol, s, e, c_lo);
            if (b == nseg - 1)
                t0[k + l] = e;
        }
    }
}

// ---------------------------------------------------------------------------
// 3. segment kernel
// ---------------------------------------------------------------------------
template <typename T>
struct SegLayout {
    static constexpr int NW = kSegThreads / 32;
    static constexpr size_t o_col = 0;
    static constexpr size_t o_val = o_col + mid_a16(kSegCap * 4);
    static constexpr size_t o_ia = o_val + mid_a16(kSegCap * sizeof(T));
    static constexpr size_t o_ib = o_ia + mid_a16(kSegCap * 2);
    static constexpr size_t o_leaf = o_ib + mid_a16(kSegCap * 2);
    static constexpr size_t o_loff = o_leaf + mid_a16(kSegCap * 2);
    static constexpr size_t o_lbs = o_loff + mid_a16((kSegCap + 1) * 4);
    static constexpr size_t o_lleaf = o_lbs + mid_a16(kSegCap * 4);
    static constexpr size_t o_rcnt = o_lleaf + mid_a16(kSegCap * 2);
    static constexpr size_t o_head = o_rcnt + mid_a16(256 * NW * 2);
    static constexpr size_t o_ws = o_head + mid_a16(kSegCap / 8 + 4);
    static constexpr size_t o_misc = o_ws + mid_a16((NW + 1) * 8);
    static constexpr size_t bytes = o_misc + 64;
};

// One stable LSD pass with 8-bit digits over u16 indices; the digit of index
// e is ((col[e] - c_lo) >> shift) & 255.  Same ownership scheme as radix_pass.
template <int NT>
__device__ __forceinline__ void radix_pass_idx(const unsigned short *__restrict__ src,
                                               unsigned short *__restrict__ dst,
                                               const int *__restrict__ col, int c_lo, int n,
                                               int shift, unsigned short *cnt, int *ws)
{
    constexpr int NW = NT / 32;
    constexpr int RADIX = 256;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int per = ((n + NW - 1) / NW + 31) & ~31;
    const int beg = min(w * per, n), end = min(beg + per, n);
    for (int d = lane; d < RADIX; d += 32)
        cnt[d * NW + w] = 0;
    __syncwarp();
    for (int base = beg; base < end; base += 32) {
        const int i = base + lane;
        const bool valid = i < end;
        const unsigned d = valid ? ((unsigned)(col[src[i]] - c_lo) >> shift) & 255u : 0xffffffffu;
        const unsigned peers = __match_any_sync(kFull, d);
        if (valid && lane == __ffs(peers) - 1)
            cnt[d * NW + w] += (unsigned short)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    constexpr int PER = RADIX * NW / NT;
    int local[PER];
    int s = 0;
#pragma unroll
    for (int j = 0; j < PER; j++) {
        local[j] = cnt[threadIdx.x * PER + j];
        s += local[j];
    }
    int tot;
    int ex = block_excl_scan<NT>(s, ws, &tot);
#pragma unroll
    for (int j = 0; j < PER; j++) {
        cnt[threadIdx.x * PER + j] = (unsigned short)ex;
        ex += local[j];
    }
    __syncthreads();
    for (int base = beg; base < end; base += 32) {
        const int i = base + lane;
        const bool valid = i < end;
        const unsigned short e = valid ? src[i] : 0;
        const unsigned d = valid ? ((unsigned)(col[e] - c_lo) >> shift) & 255u : 0xffffffffu;
        const unsigned peers = __match_any_sync(kFull, d);
        if (valid)
            dst[cnt[d * NW + w] + __popc(peers & lanemask_lt())] = e;
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1)
            cnt[d * NW + w] += (unsigned short)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
}

template <typename T, bool UPPER>
__global__ void __launch_bounds__(kSegThreads) k_seg_numeric(CsrDev A, CsrDev B, PlanDev P,
                                                             const int *crpt, int *ccol, T *cval)
{
    constexpr int NT = kSegThreads;
    using L = SegLayout<T>;
    extern __shared__ __align__(16) unsigned char smem[];
    int *col = (int *)(smem + L::o_col);
    T *val = (T *)(smem + L::o_val);
    unsigned short *ia = (unsigned short *)(smem + L::o_ia);
    unsigned short *ib = (unsigned short *)(smem + L::o_ib);
    unsigned short *leafp = (unsigned short *)(smem + L::o_leaf);
    int *loff = (int *)(smem + L::o_loff);
    int *lbs = (int *)(smem + L::o_lbs);
    unsigned short *lleaf = (unsigned short *)(smem + L::o_lleaf);
    unsigned short *rcnt = (unsigned short *)(smem + L::o_rcnt);
    unsigned *head = (unsigned *)(smem + L::o_head);
    long long *ws = (long long *)(smem + L::o_ws);
    int *wsi = (int *)(smem + L::o_ws);
    int *misc = (int *)(smem + L::o_misc);
    const int tid = threadIdx.x;
    const int nsegs = P.cnt->n_seg;
    const int *__restrict__ bcol = B.col;
    const T *__restrict__ bval = (const T *)B.val;
    const T *__restrict__ aval = (const T *)A.val;
    for (;;) {
        if (tid == 0)
            misc[0] = atomicAdd(&P.cnt->work_seg, 1);
        __syncthreads();
        const int item = misc[0];
        __syncthreads();
        if (item >= nsegs)
            break;
        const int slot = P.seg_list[item];
        const SegDesc d = P.seg[slot];
        const int row = d.row;
        const int a0 = A.rpt[row];
        const int k = A.rpt[row + 1] - a0;
        const int *sp0 = P.split + d.tab + (long long)d.bidx * k;
        const int *sp1 = sp0 + k;
        // nonempty sub-lists of the segment, in leaf order
        int lcarry = 0, pcarry = 0;
        for (int lb = 0; lb < k; lb += NT) {
            const int l = lb + tid;
            int st = 0, len = 0;
            if (l < k) {
                st = sp0[l];
                len = sp1[l] - st;
            }
            const bool ne = len > 0;
            long long tot;
            const long long ex = block_excl_scan<NT, long long>(
                ((long long)(ne ? 1 : 0) << 32) | (long long)len, ws, &tot);
            const int li = lcarry + (int)(ex >> 32);
            const int po = pcarry + (int)(ex & 0xffffffffLL);
            if (ne && li < kSegCap) {
                loff[li] = po;
                lbs[li] = st;
                lleaf[li] = (unsigned short)l;
            }
            lcarry += (int)(tot >> 32);
            pcarry += (int)(tot & 0xffffffffLL);
        }
        const int nlists = lcarry, nprod = pcarry;
        if (nprod > kSegCap || nprod != d.nprod) {
            if (tid == 0)
                atomicOr(&P.cnt->err, kErrWindowOverflow);
            continue;
        }
        if (tid == 0)
            loff[nlists] = nprod;
        for (int i = tid; i < (nprod + 31) / 32 + 1; i += NT)
            head[i] = 0;
        __syncthreads();
        const int ipt = (nprod + NT - 1) / NT;
        const int p0 = min(tid * ipt, nprod), p1 = min(p0 + ipt, nprod);
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
                        c[i] = bcol[addr[i]];
                        bv[i] = bval[addr[i]];
                        av[i] = aval[a0 + lleaf[lid[i]]];
                    }
                }
#pragma unroll
                for (int i = 0; i < kGatherBatch; i++) {
                    if (i < n) {
                        const int e = p + i;
                        col[e] = c[i];
                        val[e] = vmul(av[i], bv[i]);
                        leafp[e] = lleaf[lid[i]];
                        ia[e] = (unsigned short)e;
                    }
                }
            }
        }
        __syncthreads();
        // stable sort by column offset (list-major input order = leaf order)
        const int span = d.c_hi - d.c_lo;
        unsigned short *src = ia, *dst = ib;
        for (int sh = 0; sh < kSegSpanBits && (span - 1) >> sh; sh += 8) {
            radix_pass_idx<NT>(src, dst, col, d.c_lo, nprod, sh, rcnt, wsi);
            unsigned short *x = src;
            src = dst;
            dst = x;
        }
        // heads and their ranks
        int nh = 0;
        {
            int prev = p0 > 0 && p0 < p1 ? col[src[p0 - 1]] : -1;
            for (int p = p0; p < p1; p++) {
                const int c = col[src[p]];
                if (c != prev) {
                    atomicOr(&head[p >> 5], 1u << (p & 31));
                    nh++;
                }
                prev = c;
            }
        }
        long long htot;
        const int hx = (int)block_excl_scan<NT, long long>(nh, ws, &htot);
        const long long obase = (UPPER ? P.scan_flop[row] : (long long)crpt[row]) + d.u_off;
        {
            int h = hx;
            for (int p = p0; p < p1; p++) {
                if (!((head[p >> 5] >> (p & 31)) & 1u))
                    continue;
                const int e = src[p];
                int q = p + 1;
                T v;
                if (q >= nprod || ((head[q >> 5] >> (q & 31)) & 1u)) {
                    v = val[e];
                } else {
                    ShiftReduce<T> sr;
                    sr.init(leafp[e], val[e]);
                    for (; q < nprod && !((head[q >> 5] >> (q & 31)) & 1u); q++) {
                        const int e2 = src[q];
                        sr.push(leafp[e2], val[e2]);
                    }
                    v = sr.finish();
                }
                ccol[obase + h] = col[e];
                cval[obase + h] = v;
                h++;
            }
        }
        if (tid == 0) {
            // the segment must produce exactly its share of the row's columns
            const int nseg = P.seg_n[row];
            const int next_u = (d.bidx + 1 < nseg) ? P.seg[slot + 1].u_off : P.nnz[row];
            if ((int)htot != next_u - d.u_off)
                atomicOr(&P.cnt->err, kErrNnzMismatch);
        }
        __syncthreads();
    }
}

}  // namespace brm
