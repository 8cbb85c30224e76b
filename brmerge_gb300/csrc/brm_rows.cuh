// brm_rows.cuh -- symbolic and numeric row kernels of BRMerge SpGEMM.
//
// Semantics (BRMerge-SpGEMM/inc/spgemm.h:580-721).  Row i of C is the binary
// merge of k lists, list l being row acol[arpt[i]+l] of B scaled by
// aval[arpt[i]+l]; adjacent lists merge pairwise level by level and equal
// columns add as left + right.  Per output column that is a binary trie over
// the leaf index l (ShiftReduce in brm_common.cuh).  The kernels below do not
// replay the merge levels; they compute the same values in a GPU-friendly
// order of work:
//
//   * structure: a bitmap of the row's columns in shared memory gives every
//     column its output rank (prefix popcount), so positions are known
//     without merging (exact nnz, spgemm.h:505-562, comes from the popcount);
//   * order: the products of a window are sorted by (rank, original position)
//     with a stable block radix sort; the original position is list-major, so
//     each column's contributions come out in increasing leaf order and one
//     thread per column evaluates the trie with ShiftReduce;
//   * size: columns are processed in chunks of kChunkBits and the products of
//     a chunk in windows of at most kCap, cut at 32-column word boundaries.
//
// Rows whose lists do not fit the shared-memory tables (more than kLMax lists,
// or more than kCap products inside one 32-column word) take the spill path,
// a per-row merge in global scratch memory.
#pragma once

#include <climits>

#include "brm_check.cuh"
#include "brm_common.cuh"
#include "brm_plan.h"

namespace brm {

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------

// Threads per list for a loop over the elements of many lists: about the
// average list length, a power of two in [1, 32].
__device__ __forceinline__ int group_size(long long elems, int lists)
{
    long long avg = lists > 0 ? elems / lists : elems;
    int g = 1;
    while (g < 32 && (long long)(g * 2) <= avg)
        g <<= 1;
    return g;
}

// Number of entries in the sorted col[s..e) that are < key (galloping search).
__device__ __forceinline__ int gallop_count(const int *__restrict__ col, int s, int e, int key)
{
    if (s >= e || col[s] >= key)
        return 0;
    int lo = s, step = 1;
    while (lo + step < e && col[lo + step] < key) {
        lo += step;
        step <<= 1;
    }
    int hi = min(lo + step, e);
    while (hi - lo > 1) {
        int mid = lo + ((hi - lo) >> 1);
        if (col[mid] < key)
            lo = mid;
        else
            hi = mid;
    }
    return hi - s;
}

// First index in the sorted col[s..e) whose value is >= key.
__device__ __forceinline__ int lower_bound_idx(const int *__restrict__ col, int s, int e, int key)
{
    while (s < e) {
        int mid = s + ((e - s) >> 1);
        if (col[mid] < key)
            s = mid + 1;
        else
            e = mid;
    }
    return s;
}

// Smallest set bit index >= from in the bitset, or nw if none below nw.
__device__ __forceinline__ int next_set_bit(const unsigned *bits, int from, int nw)
{
    int w = from;
    while (w < nw) {
        unsigned word = bits[w >> 5] >> (w & 31);
        if (word) {
            int r = w + __ffs(word) - 1;
            return r < nw ? r : nw;
        }
        w = (w | 31) + 1;
    }
    return nw;
}

// One stable LSD pass of a block radix sort over keys src[0..n): the digit is
// bits [shift, shift+bits) of the key.  Each warp owns a contiguous slice of
// the input, so (digit, warp, lane) order is input order and the pass is
// stable.  cnt holds (1<<kRadixBits) * NW 16-bit counters, digit-major.
template <int NT>
__device__ __forceinline__ void radix_pass(const unsigned *__restrict__ src, unsigned *__restrict__ dst,
                                           int n, int shift, int bits, unsigned short *cnt,
                                           int *ws)
{
    constexpr int NW = NT / 32;
    constexpr int RADIX = 1 << kRadixBits;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned mask = (1u << bits) - 1u;
    const int per = ((n + NW - 1) / NW + 31) & ~31;
    const int beg = min(w * per, n), end = min(beg + per, n);
    for (int d = lane; d < RADIX; d += 32)
        cnt[d * NW + w] = 0;
    __syncwarp();
    for (int base = beg; base < end; base += 32) {
        int i = base + lane;
        bool valid = i < end;
        unsigned d = valid ? (src[i] >> shift) & mask : 0xffffffffu;
        unsigned peers = __match_any_sync(kFull, d);
        if (valid && lane == __ffs(peers) - 1)
            cnt[d * NW + w] += (unsigned short)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // exclusive scan of the counters in (digit, warp) order
    constexpr int PER = RADIX * NW / NT;  // counters per thread
    static_assert(RADIX * NW % NT == 0, "counter layout");
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
        int i = base + lane;
        bool valid = i < end;
        unsigned key = valid ? src[i] : 0u;
        unsigned d = valid ? (key >> shift) & mask : 0xffffffffu;
        unsigned peers = __match_any_sync(kFull, d);
        if (valid) {
            int rank = __popc(peers & lanemask_lt());
            dst[cnt[d * NW + w] + rank] = key;
        }
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1)
            cnt[d * NW + w] += (unsigned short)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Shared-memory layout of the numeric row CTA (dynamic shared memory).
// ---------------------------------------------------------------------------
template <typename T>
struct NumLayout {
    static constexpr int NW = kRowThreads / 32;
    static constexpr size_t a16(size_t x) { return (x + 15) & ~size_t(15); }
    static constexpr size_t o_bm = 0;
    static constexpr size_t o_aux = o_bm + a16(kChunkWords * 4);
    static constexpr size_t o_wst = o_aux + a16((kChunkWords + 1) * 4);
    static constexpr size_t o_lcur = o_wst + a16(kChunkWords / 32 * 4);
    static constexpr size_t o_lend = o_lcur + a16(kLMax * 4);
    static constexpr size_t o_loff = o_lend + a16(kLMax * 4);
    static constexpr size_t o_pval = o_loff + a16((kLMax + 1) * 4);
    static constexpr size_t o_keyA = o_pval + a16(kCap * sizeof(T));
    static constexpr size_t o_keyB = o_keyA + a16((kCap + 1) * 4);
    static constexpr size_t o_ocol = o_keyB + a16((kCap + 1) * 4);
    static constexpr size_t o_leaf = o_ocol + a16(kCap * 4);
    static constexpr size_t o_rcnt = o_leaf + a16(kCap * 2);
    static constexpr size_t o_ws = o_rcnt + a16((1 << kRadixBits) * NW * 2);
    static constexpr size_t o_misc = o_ws + a16((NW + 1) * 8);
    static constexpr size_t bytes = o_misc + 64;
};

struct SymLayout {
    static constexpr int NW = kRowThreads / 32;
    static constexpr size_t o_bm = 0;
    static constexpr size_t o_aux = o_bm + kChunkWords * 4;
    static constexpr size_t o_ws = o_aux + kChunkWords * 4;
    static constexpr size_t o_misc = o_ws + (NW + 1) * 8;
    static constexpr size_t bytes = o_misc + 64;
};

// Scratch bytes reserved for one spill row (two ping-pong product buffers and
// two list-offset arrays, values sized as double for both value types).
__host__ __device__ __forceinline__ unsigned long long spill_row_bytes(long long flop, int k)
{
    unsigned long long b = (unsigned long long)flop * (4 + 4 + 8 + 8) + (unsigned long long)(k + 1) * 8;
    return (b + 255) & ~255ull;
}

// ---------------------------------------------------------------------------
// Symbolic row CTA: exact nnz per row by bitmap popcount; flags spill rows.
// ---------------------------------------------------------------------------
template <bool ONLY_HEAVY>
__global__ void __launch_bounds__(kRowThreads) k_rows_symbolic(CsrDev A, CsrDev B, PlanDev P)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    constexpr int NT = kRowThreads;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned *bm = (unsigned *)(smem + SymLayout::o_bm);
    unsigned *hist = (unsigned *)(smem + SymLayout::o_aux);
    long long *ws = (long long *)(smem + SymLayout::o_ws);
    int *misc = (int *)(smem + SymLayout::o_misc);
    const int tid = threadIdx.x;
    const int M = A.M;
    const int nheavy = 0;  // heavy rows are segmented (brm_seg.cuh); this kernel takes kBinMid
    const int ntot = nheavy + P.cnt->bin_count[kBinMid];
    const int *heavy = P.rows + (size_t)kBinHeavy * M;
    const int *mid = P.rows + (size_t)kBinMid * M;
    const int *__restrict__ bcol = B.col;

    for (;;) {
        if (tid == 0)
            misc[0] = atomicAdd(&P.cnt->work_sym, 1);
        __syncthreads();
        const int item = misc[0];
        __syncthreads();
        if (item >= ntot)
            break;
        const int row = item < nheavy ? heavy[item] : mid[item - nheavy];
        const int a0 = A.rpt[row];
        const int k = A.rpt[row + 1] - a0;
        const int F = P.flop[row];
        const bool need_hist = F > kCap;
        if (ONLY_HEAVY && !need_hist && k <= kLMax)
            continue;

        int mn = INT_MAX, mx = -1;
        for (int l = tid; l < k; l += NT) {
            int b = A.col[a0 + l];
            if ((unsigned)b >= (unsigned)B.M)
                continue;
            int s = B.rpt[b], e = B.rpt[b + 1];
            if (s < e) {
                mn = min(mn, bcol[s]);
                mx = max(mx, bcol[e - 1]);
            }
        }
        mn = (int)block_min<NT, long long>(mn, ws);
        mx = (int)block_max<NT, long long>(mx, ws);
        if (mn < 0 || mx >= B.N) {
            if (tid == 0)
                atomicOr(&P.cnt->err, kErrBadInput);
            continue;
        }
        const int G = group_size(F, k);
        const int lg = tid & (G - 1);
        long long count = 0;
        unsigned maxh = 0;
        for (long long clo = mn; clo <= mx; clo += kChunkBits) {
            const int lo = (int)clo;
            const int chi = (int)min((long long)mx + 1, clo + kChunkBits);
            const int span = chi - lo;
            const int nw = (span + 31) >> 5;
            const bool multi = (long long)mx + 1 - mn > kChunkBits;
            for (int i = tid; i < nw; i += NT) {
                bm[i] = 0;
                if (need_hist)
                    hist[i] = 0;
            }
            __syncthreads();
            for (int l = tid / G; l < k; l += NT / G) {
                int b = A.col[a0 + l];
                if ((unsigned)b >= (unsigned)B.M)
                    continue;
                int s = B.rpt[b], e = B.rpt[b + 1];
                if (multi) {
                    s = lower_bound_idx(bcol, s, e, lo);
                    e = lower_bound_idx(bcol, s, e, chi);
                }
                for (int idx = s + lg; idx < e; idx += G) {
                    int rc = bcol[idx] - lo;
                    if ((unsigned)rc < (unsigned)span) {
                        atomicOr(&bm[rc >> 5], 1u << (rc & 31));
                        if (need_hist)
                            atomicAdd(&hist[rc >> 5], 1u);
                    } else {
                        atomicOr(&P.cnt->err, kErrBadInput);
                    }
                }
            }
            __syncthreads();
            long long c = 0;
            unsigned h = 0;
            for (int i = tid; i < nw; i += NT) {
                c += __popc(bm[i]);
                if (need_hist)
                    h = max(h, hist[i]);
            }
            count += block_sum<NT, long long>(c, ws);
            if (need_hist)
                maxh = max(maxh, (unsigned)block_max<NT, long long>((long long)h, ws));
            __syncthreads();
        }
        if (tid == 0) {
            if (!ONLY_HEAVY)
                P.nnz[row] = (int)count;
            if (k > kLMax || maxh > (unsigned)kCap) {
                P.spill[row] = 1;
                int idx = atomicAdd(&P.cnt->spill_count, 1);
                P.spill_rows[idx] = row;
                P.spill_off[idx] = atomicAdd(&P.cnt->spill_bytes, spill_row_bytes(F, k));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Numeric row CTA.
// ---------------------------------------------------------------------------
template <typename T, bool UPPER>
__device__ __forceinline__ void numeric_row(const CsrDev &A, const CsrDev &B, const PlanDev &P,
                                            int row, long long out_base, int expect, int *ccol,
                                            T *cval, unsigned char *smem)
{
    constexpr int NT = kRowThreads;
    using L = NumLayout<T>;
    unsigned *bm = (unsigned *)(smem + L::o_bm);
    unsigned *aux = (unsigned *)(smem + L::o_aux);
    unsigned *wst = (unsigned *)(smem + L::o_wst);
    int *lcur = (int *)(smem + L::o_lcur);
    int *lend = (int *)(smem + L::o_lend);
    int *loff = (int *)(smem + L::o_loff);
    T *pval = (T *)(smem + L::o_pval);
    unsigned *keyA = (unsigned *)(smem + L::o_keyA);
    unsigned *keyB = (unsigned *)(smem + L::o_keyB);
    int *ocol = (int *)(smem + L::o_ocol);
    unsigned short *pleaf = (unsigned short *)(smem + L::o_leaf);
    unsigned short *rcnt = (unsigned short *)(smem + L::o_rcnt);
    long long *ws = (long long *)(smem + L::o_ws);
    int *wsi = (int *)(smem + L::o_ws);
    volatile int *wflag = (int *)(smem + L::o_misc) + 1;  // set when a guard trips
    const int tid = threadIdx.x;
    const int *__restrict__ bcol = B.col;
    const T *__restrict__ bval = (const T *)B.val;
    const T *__restrict__ aval = (const T *)A.val;

    const int a0 = A.rpt[row];
    const int k = A.rpt[row + 1] - a0;
    const int F = P.flop[row];

    // list table and the row's column range
    int mn = INT_MAX, mx = -1;
    for (int l = tid; l < k; l += NT) {
        int b = A.col[a0 + l];
        int s = 0, e = 0;
        if ((unsigned)b < (unsigned)B.M) {
            s = B.rpt[b];
            e = B.rpt[b + 1];
        }
        lcur[l] = s;
        lend[l] = e;
        if (s < e) {
            mn = min(mn, bcol[s]);
            mx = max(mx, bcol[e - 1]);
        }
    }
    mn = (int)block_min<NT, long long>(mn, ws);
    mx = (int)block_max<NT, long long>(mx, ws);
    if (mx < 0 || mn < 0 || mx >= B.N) {
        if (tid == 0) {
            if (mx >= 0)
                atomicOr(&P.cnt->err, kErrBadInput);
            if (UPPER)
                P.nnz[row] = 0;
        }
        __syncthreads();
        return;
    }
    const bool multi = (long long)mx + 1 - mn > kChunkBits;
    const int lpt = (k + NT - 1) / NT;  // lists per thread (contiguous) for scans
    int written = 0;
    bool failed = false;

    for (long long clo = mn; clo <= mx && !failed; clo += kChunkBits) {
        const int lo = (int)clo;
        const int chi = (int)min((long long)mx + 1, clo + kChunkBits);
        const int span = chi - lo;
        const int nw = (span + 31) >> 5;
        for (int i = tid; i < nw; i += NT) {
            bm[i] = 0;
            aux[i] = 0;
        }
        for (int i = tid; i < (nw + 31) / 32; i += NT)
            wst[i] = 0;
        if (multi) {
            // limit every list to the chunk: lend = first index with col >= chi
            for (int l = tid; l < k; l += NT) {
                int b = A.col[a0 + l];
                int e = ((unsigned)b < (unsigned)B.M) ? B.rpt[b + 1] : lcur[l];
                lend[l] = lower_bound_idx(bcol, lcur[l], e, chi);
            }
        }
        __syncthreads();
        // pass A: column bitmap and products per 32-column word
        long long fchunk_local = 0;
        {
            const int G = group_size(F, k);
            const int lg = tid & (G - 1);
            for (int l = tid / G; l < k; l += NT / G) {
                const int s = lcur[l], e = lend[l];
                if (lg == 0)
                    fchunk_local += e - s;
                for (int idx = s + lg; idx < e; idx += G) {
                    int rc = bcol[idx] - lo;
                    if ((unsigned)rc < (unsigned)span) {
                        atomicOr(&bm[rc >> 5], 1u << (rc & 31));
                        atomicAdd(&aux[rc >> 5], 1u);
                    } else {
                        atomicOr(&P.cnt->err, kErrBadInput);
                    }
                }
            }
        }
        const long long fchunk = block_sum<NT, long long>(fchunk_local, ws);
        const bool one_window = fchunk <= kCap;
        // per-word scan of (products, distinct columns); window starts; rank table
        {
            const int wpt = (nw + NT - 1) / NT;
            const int w0 = min(tid * wpt, nw), w1 = min(w0 + wpt, nw);
            unsigned long long sp = 0;
            for (int w = w0; w < w1; w++)
                sp += ((unsigned long long)aux[w] << 32) | (unsigned)__popc(bm[w]);
            const unsigned prevh = (w0 > 0 && w0 < nw) ? aux[w0 - 1] : 0u;
            long long tot;
            long long ex = block_excl_scan<NT, long long>((long long)sp, ws, &tot);
            unsigned long long run = (unsigned long long)ex;
            unsigned ph = prevh;
            constexpr unsigned Tcut = kCap / 2;
            for (int w = w0; w < w1; w++) {
                const unsigned h = aux[w];
                const unsigned pe = (unsigned)(run >> 32);  // products before word w
                if (!one_window) {
                    bool start = (w == 0) || h > Tcut || ph > Tcut ||
                                 (pe / Tcut) != ((pe - ph) / Tcut);
                    if (start)
                        atomicOr(&wst[w >> 5], 1u << (w & 31));
                    if (h > (unsigned)kCap)
                        atomicOr(&P.cnt->err, kErrWindowOverflow);
                }
                aux[w] = (unsigned)(run & 0xffffffffu);  // distinct columns before word w
                run += ((unsigned long long)h << 32) | (unsigned)__popc(bm[w]);
                ph = h;
            }
            if (tid == 0)
                aux[nw] = (unsigned)((unsigned long long)tot & 0xffffffffu);
        }
        __syncthreads();

        int w0 = 0;
        while (w0 < nw) {
            const int w1 = one_window ? nw : next_set_bit(wst, w0 + 1, nw);
            const int c_hi = (w1 == nw) ? chi : lo + 32 * w1;
            const int ubase = (int)aux[w0];
            const int Uw = (int)aux[w1] - ubase;
            const bool last = (w1 == nw);
            // products of every list inside the window, and their offsets
            if (tid == 0)
                *wflag = 0;  // ordered before the guards by the scan's barriers
            int sum = 0;
            {
                const int l0 = min(tid * lpt, k), l1 = min(l0 + lpt, k);
                for (int l = l0; l < l1; l++) {
                    int s = lcur[l], e = lend[l];
                    int c = last ? e - s : gallop_count(bcol, s, e, c_hi);
                    loff[l] = c;
                    sum += c;
                }
                int tot;
                int base = block_excl_scan<NT, int>(sum, wsi, &tot);
                for (int l = l0; l < l1; l++) {
                    int c = loff[l];
                    loff[l] = base;
                    base += c;
                }
                if (tid == 0)
                    loff[k] = tot;
                __syncthreads();
            }
            const int Fw = loff[k];
            if (Fw > kCap || Uw > Fw) {
                if (tid == 0)
                    atomicOr(&P.cnt->err, kErrWindowOverflow);
                failed = true;
                break;
            }
            // stage the window's products: key = (rank << 16) | position
            {
                const int G = group_size(Fw, k);
                const int lg = tid & (G - 1);
                for (int l = tid / G; l < k; l += NT / G) {
                    const int s = lcur[l];
                    const int base = loff[l];
                    const int n = loff[l + 1] - base;
                    if (n == 0)
                        continue;
                    const T av = aval[a0 + l];
                    for (int q = lg; q < n; q += G) {
                        const int idx = s + q;
                        const int c = bcol[idx];
                        const T v = vmul(av, bval[idx]);
                        const int e = base + q;
                        const int rc = c - lo;
                        if ((unsigned)rc >= (unsigned)span) {
                            atomicOr(&P.cnt->err, kErrBadInput);
                            *wflag = 1;
                            continue;
                        }
                        const int w = rc >> 5;
                        const int u = (int)aux[w] + __popc(bm[w] & ((1u << (rc & 31)) - 1u)) - ubase;
                        if ((unsigned)u >= (unsigned)Uw) {
                            atomicOr(&P.cnt->err, kErrWindowOverflow);
                            *wflag = 1;
                            continue;
                        }
                        keyA[e] = ((unsigned)u << 16) | (unsigned)e;
                        pleaf[e] = (unsigned short)l;
                        pval[e] = v;
                        ocol[u] = c;
                    }
                }
            }
            __syncthreads();
            if (*wflag) {  // a staged key is missing: do not sort or index with it
                failed = true;
                break;
            }
            const bool nodup = (Fw == Uw);
            const unsigned *R = keyA;
            unsigned *S = keyB;
            if (nodup) {
                for (int e = tid; e < Fw; e += NT)
                    keyB[keyA[e] >> 16] = (unsigned)e;
            } else {
                const int nb = Uw > 1 ? 32 - __clz(Uw - 1) : 0;
                unsigned *src = keyA, *dst = keyB;
                for (int sh = 0; sh < nb; sh += kRadixBits) {
                    radix_pass<NT>(src, dst, Fw, 16 + sh, min(kRadixBits, nb - sh), rcnt, wsi);
                    unsigned *t = src;
                    src = dst;
                    dst = t;
                }
                R = src;
                S = dst;
                for (int i = tid; i < Fw; i += NT) {
                    unsigned u = R[i] >> 16;
                    if (i == 0 || (R[i - 1] >> 16) != u)
                        S[u] = (unsigned)i;
                }
            }
            __syncthreads();
            // one thread per output column: order-exact reduction, coalesced store
            for (int u = tid; u < Uw; u += NT) {
                T v;
                if (nodup) {
                    v = pval[S[u]];
                } else {
                    const int i0 = (int)S[u];
                    const int i1 = (u + 1 < Uw) ? (int)S[u + 1] : Fw;
                    int e = (int)(R[i0] & 0xffffu);
                    if (i1 - i0 == 1) {
                        v = pval[e];
                    } else {
                        ShiftReduce<T> sr;
                        sr.init(pleaf[e], pval[e]);
                        for (int i = i0 + 1; i < i1; i++) {
                            e = (int)(R[i] & 0xffffu);
                            sr.push(pleaf[e], pval[e]);
                        }
                        v = sr.finish();
                    }
                }
                const long long o = out_base + written + u;
                if (BRM_IN(P.cnt, o, P.c_cap)) {
                    ccol[o] = ocol[u];
                    cval[o] = v;
                }
            }
            written += Uw;
            {
                const int l0 = min(tid * lpt, k), l1 = min(l0 + lpt, k);
                for (int l = l0; l < l1; l++)
                    lcur[l] += loff[l + 1] - loff[l];
            }
            __syncthreads();
            w0 = w1;
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (UPPER)
            P.nnz[row] = written;
        else if (!failed && written != expect)
            atomicOr(&P.cnt->err, kErrNnzMismatch);
    }
    __syncthreads();
}

template <typename T, bool UPPER>
__global__ void __launch_bounds__(kRowThreads, 1)
    k_rows_numeric(CsrDev A, CsrDev B, PlanDev P, const int *crpt, int *ccol, T *cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    extern __shared__ __align__(16) unsigned char smem[];
    int *misc = (int *)(smem + NumLayout<T>::o_misc);
    const int M = A.M;
    const int nheavy = 0;  // heavy rows are segmented (brm_seg.cuh); this kernel takes kBinMid
    const int ntot = nheavy + P.cnt->bin_count[kBinMid];
    const int *heavy = P.rows + (size_t)kBinHeavy * M;
    const int *mid = P.rows + (size_t)kBinMid * M;
    for (;;) {
        if (threadIdx.x == 0)
            misc[0] = atomicAdd(&P.cnt->work_num, 1);
        __syncthreads();
        const int item = misc[0];
        __syncthreads();
        if (item >= ntot)
            break;
        const int row = item < nheavy ? heavy[item] : mid[item - nheavy];
        if (P.spill[row] || row < P.r_lo || row >= P.r_hi)
            continue;
        long long base;
        int expect = 0;
        if (UPPER) {
            base = P.scan_flop[row];
        } else {
            base = crpt[row];
            expect = crpt[row + 1] - crpt[row];
        }
        numeric_row<T, UPPER>(A, B, P, row, base, expect, ccol, cval, smem);
    }
}

// ---------------------------------------------------------------------------
// Warp kernels: rows with at most 32 products and >= 2 nonempty lists.
// Lane e holds product e (list-major order); symbolic counts distinct columns
// with match_any; numeric sorts the lanes by (column, leaf) and evaluates the
// merge trie level by level (siblings 2m and 2m+1 are adjacent once sorted).
// ---------------------------------------------------------------------------
template <typename T, bool NUMERIC>
__device__ __forceinline__ int warp_gather(const CsrDev &A, const CsrDev &B, int a0, int k,
                                           int &my_col, int &my_leaf, T &my_val)
{
    const int lane = threadIdx.x & 31;
    my_col = INT_MAX;
    my_leaf = 0;
    my_val = T(0);
    int filled = 0;
    for (int lb = 0; lb < k; lb += 32) {
        const int l = lb + lane;
        int s = 0, len = 0;
        if (l < k) {
            int b = A.col[a0 + l];
            if ((unsigned)b < (unsigned)B.M) {
                s = B.rpt[b];
                len = B.rpt[b + 1] - s;
            }
        }
        const int incl = warp_incl_scan(len);
        const int excl = incl - len;
        const int tot = __shfl_sync(kFull, incl, 31);
        unsigned mask = __ballot_sync(kFull, len > 0);
        while (mask) {
            const int src = __ffs(mask) - 1;
            mask &= mask - 1;
            const int ls = __shfl_sync(kFull, s, src);
            const int ll = __shfl_sync(kFull, len, src);
            const int lo = __shfl_sync(kFull, excl, src) + filled;
            if (lane >= lo && lane < lo + ll) {
                const int idx = ls + (lane - lo);
                my_col = B.col[idx];
                my_leaf = lb + src;
                if (NUMERIC)
                    my_val = vmul(((const T *)A.val)[a0 + lb + src], ((const T *)B.val)[idx]);
            }
        }
        filled += tot;
    }
    return filled;
}

template <int UNUSED = 0>
__global__ void __launch_bounds__(256) k_warp_symbolic(CsrDev A, CsrDev B, PlanDev P)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int n = P.cnt->bin_count[kBinWarp];
    const int *rows = P.rows + (size_t)kBinWarp * A.M;
    for (int it = gw; it < n; it += nwarps) {
        const int row = rows[it];
        const int a0 = A.rpt[row], k = A.rpt[row + 1] - a0;
        int c, leaf;
        double v;
        const int f = warp_gather<double, false>(A, B, a0, k, c, leaf, v);
        const bool valid = lane < f;
        const unsigned peers = __match_any_sync(kFull, c);
        const unsigned uniq = __ballot_sync(kFull, valid && lane == __ffs(peers) - 1);
        if (lane == 0)
            P.nnz[row] = __popc(uniq);
    }
}

template <typename T, bool UPPER>
__global__ void __launch_bounds__(256) k_warp_numeric(CsrDev A, CsrDev B, PlanDev P,
                                                      const int *crpt, int *ccol, T *cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int n = P.cnt->bin_count[kBinWarp];
    const int *rows = P.rows + (size_t)kBinWarp * A.M;
    for (int it = gw; it < n; it += nwarps) {
        const int row = rows[it];
        if (row < P.r_lo || row >= P.r_hi)
            continue;
        const int a0 = A.rpt[row], k = A.rpt[row + 1] - a0;
        int c, leaf;
        T v;
        const int f = warp_gather<T, true>(A, B, a0, k, c, leaf, v);
        const bool valid = lane < f;
        unsigned long long key =
            valid ? (((unsigned long long)(unsigned)c << 32) | (unsigned)leaf) : ~0ull;
        // bitonic sort of (key, value) across the warp, ascending
#pragma unroll
        for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                unsigned long long ok = __shfl_xor_sync(kFull, key, stride);
                T ov = __shfl_xor_sync(kFull, v, stride);
                const bool up = (lane & size) == 0 || size == 32;
                const bool lower = (lane & stride) == 0;
                const bool take = (lower == up) ? (ok < key) : (ok > key);
                if (take) {
                    key = ok;
                    v = ov;
                }
            }
        }
        c = (int)(key >> 32);
        int node = (int)(key & 0xffffffffu);
        bool active = valid;
        // level-synchronous trie reduction
        for (int lvl = 0; lvl < 31; lvl++) {
            const unsigned act = __ballot_sync(kFull, active);
            const unsigned higher = lane == 31 ? 0u : (act & (0xffffffffu << (lane + 1)));
            const int nxt = higher ? __ffs(higher) - 1 : lane;
            const int ncol = __shfl_sync(kFull, c, nxt);
            const int nnode = __shfl_sync(kFull, node, nxt);
            const T nval = __shfl_sync(kFull, v, nxt);
            const bool same = active && nxt != lane && ncol == c;
            if (!__any_sync(kFull, same))
                break;
            const bool combine = same && (node & 1) == 0 && nnode == node + 1;
            const unsigned cmask = __ballot_sync(kFull, combine);
            const unsigned lower = act & lanemask_lt();
            const int prev = lower ? 31 - __clz(lower) : -1;
            const bool absorbed = prev >= 0 && ((cmask >> prev) & 1u);
            if (combine)
                v = vadd(v, nval);
            if (absorbed)
                active = false;
            node >>= 1;
        }
        const unsigned outm = __ballot_sync(kFull, active);
        const long long base = UPPER ? P.scan_flop[row] : (long long)crpt[row];
        if (active) {
            const long long o = base + __popc(outm & lanemask_lt());
            if (BRM_IN(P.cnt, o, P.c_cap)) {
                ccol[o] = c;
                cval[o] = v;
            }
        }
        if (lane == 0) {
            if (UPPER)
                P.nnz[row] = __popc(outm);
            else if (__popc(outm) != crpt[row + 1] - crpt[row])
                atomicOr(&P.cnt->err, kErrNnzMismatch);
        }
    }
}

// ---------------------------------------------------------------------------
// Copy rows: exactly one nonempty list, C row = a * B row (every merge level
// passes the single list through unchanged).
// ---------------------------------------------------------------------------
template <typename T, bool UPPER>
__global__ void __launch_bounds__(256) k_copy_numeric(CsrDev A, CsrDev B, PlanDev P,
                                                      const int *crpt, int *__restrict__ ccol,
                                                      T *__restrict__ cval)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int n = P.cnt->bin_count[kBinCopy];
    const int *rows = P.rows + (size_t)kBinCopy * A.M;
    for (int it = gw; it < n; it += nwarps) {
        const int row = rows[it];
        if (row < P.r_lo || row >= P.r_hi)
            continue;
        const int j = A.rpt[row] + P.copy_leaf[row];
        const int b = A.col[j];
        const T a = ((const T *)A.val)[j];
        const int s = B.rpt[b];
        int len = B.rpt[b + 1] - s;
        const long long base = UPPER ? P.scan_flop[row] : (long long)crpt[row];
        if (len > 0 && !(BRM_IN(P.cnt, base + len - 1, P.c_cap) &&
                         BRM_IN(P.cnt, (long long)s + len - 1, B.nnz)))
            len = 0;  // checked build: a row outside C or B is skipped
        const int *__restrict__ bcol = B.col;
        const T *__restrict__ bval = (const T *)B.val;
        // four elements per lane in flight before the stores
        int q = lane;
        for (; q + 96 < len; q += 128) {
            int c[4];
            T v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                c[u] = bcol[s + q + 32 * u];
                v[u] = bval[s + q + 32 * u];
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                ccol[base + q + 32 * u] = c[u];
                cval[base + q + 32 * u] = vmul(a, v[u]);
            }
        }
        for (; q < len; q += 32) {
            ccol[base + q] = bcol[s + q];
            cval[base + q] = vmul(a, bval[s + q]);
        }
    }
}

// ---------------------------------------------------------------------------
// Spill path: the reference merge replayed in global scratch memory, one
// thread per row (rows with more lists or denser columns than the shared
// memory tables hold).
// ---------------------------------------------------------------------------
template <typename T, bool UPPER>
__global__ void __launch_bounds__(32) k_spill_numeric(CsrDev A, CsrDev B, PlanDev P,
                                                      const int *crpt, int *ccol, T *cval,
                                                      unsigned char *scratch,
                                                      unsigned long long scratch_bytes)
{
    if (P.cnt->abort)  // a capacity check of a captured pipeline failed
        return;
    if (threadIdx.x != 0)
        return;
    const int n = P.cnt->spill_count;
    for (int it = blockIdx.x; it < n; it += gridDim.x) {
        const int row = P.spill_rows[it];
        if (row < P.r_lo || row >= P.r_hi)
            continue;
        const int a0 = A.rpt[row], k = A.rpt[row + 1] - a0;
        const long long F = P.flop[row];
        const unsigned long long off = P.spill_off[it];
        if (off + spill_row_bytes(F, k) > scratch_bytes) {
            atomicOr(&P.cnt->err, kErrSpillCapacity);
            continue;
        }
        unsigned char *base = scratch + off;
        int *col[2];
        T *val[2];
        int *lo[2];
        col[0] = (int *)base;
        col[1] = col[0] + F;
        val[0] = (T *)(base + F * 8);
        val[1] = (T *)(base + F * 8 + F * 8);
        lo[0] = (int *)(base + F * 24);
        lo[1] = lo[0] + (k + 1);
        int nl = 0, w = 0;
        lo[0][0] = 0;
        for (int j = a0; j < a0 + k; j++) {
            const int b = A.col[j];
            const T a = ((const T *)A.val)[j];
            if ((unsigned)b < (unsigned)B.M) {
                for (int q = B.rpt[b]; q < B.rpt[b + 1]; q++) {
                    col[0][w] = B.col[q];
                    val[0][w] = vmul(a, ((const T *)B.val)[q]);
                    w++;
                }
            }
            lo[0][++nl] = w;
        }
        int src = 0;
        while (nl > 1) {
            const int dst = src ^ 1;
            int outl = 0;
            w = 0;
            lo[dst][0] = 0;
            for (int l = 0; l < nl; l += 2) {
                int p = lo[src][l], pe = lo[src][l + 1];
                if (l + 1 < nl) {
                    int q = lo[src][l + 1], qe = lo[src][l + 2];
                    while (p < pe && q < qe) {
                        const int cp = col[src][p], cq = col[src][q];
                        if (cp == cq) {
                            col[dst][w] = cp;
                            val[dst][w++] = vadd(val[src][p++], val[src][q++]);
                        } else if (cp < cq) {
                            col[dst][w] = cp;
                            val[dst][w++] = val[src][p++];
                        } else {
                            col[dst][w] = cq;
                            val[dst][w++] = val[src][q++];
                        }
                    }
                    while (q < qe) {
                        col[dst][w] = col[src][q];
                        val[dst][w++] = val[src][q++];
                    }
                }
                while (p < pe) {
                    col[dst][w] = col[src][p];
                    val[dst][w++] = val[src][p++];
                }
                lo[dst][++outl] = w;
            }
            nl = outl;
            src = dst;
        }
        const int len = nl == 1 ? lo[src][1] : 0;
        const long long ob = UPPER ? P.scan_flop[row] : (long long)crpt[row];
        for (int q = 0; q < (len > 0 && BRM_IN(P.cnt, ob + len - 1, P.c_cap) ? len : 0); q++) {
            ccol[ob + q] = col[src][q];
            cval[ob + q] = val[src][q];
        }
        if (UPPER)
            P.nnz[row] = len;
        else if (len != crpt[row + 1] - crpt[row])
            atomicOr(&P.cnt->err, kErrNnzMismatch);
    }
}

}  // namespace brm
