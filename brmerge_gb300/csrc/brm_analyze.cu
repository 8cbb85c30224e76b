// brm_analyze.cu -- row analysis, device scans, Upper compaction, validation.
#include <algorithm>
#include <climits>

#include "brm_check.cuh"
#include "brm_common.cuh"
#include "brm_kernels.h"

namespace brm {

// ---------------------------------------------------------------------------
// Row analysis.  Replaces compute_flop (spgemm.h:31-56) and the flop-balanced
// static row ranges (spgemm.h:496-503): on the GPU the balance comes from
// binning rows by their product count and handing heavy rows out first.
// A group of lanes per row; each block appends its rows to the bin lists with one
// global atomic per bin.
// ---------------------------------------------------------------------------
constexpr int kAnaThreads = 256;
constexpr int kAnaRowsPerGroup = 2;

// Reductions over a group of TW lanes (TW a power of two <= 32, the group
// aligned in the warp); `gm` is the group's lane mask.
template <int TW, typename T>
__device__ __forceinline__ T grp_sum(T v, unsigned gm)
{
#pragma unroll
    for (int o = TW / 2; o > 0; o >>= 1)
        v += __shfl_xor_sync(gm, v, o);
    return v;
}
template <int TW, typename T>
__device__ __forceinline__ T grp_max(T v, unsigned gm)
{
#pragma unroll
    for (int o = TW / 2; o > 0; o >>= 1) {
        const T n = __shfl_xor_sync(gm, v, o);
        v = n > v ? n : v;
    }
    return v;
}
template <int TW, typename T>
__device__ __forceinline__ T grp_min(T v, unsigned gm)
{
#pragma unroll
    for (int o = TW / 2; o > 0; o >>= 1) {
        const T n = __shfl_xor_sync(gm, v, o);
        v = n < v ? n : v;
    }
    return v;
}

// A group of TW lanes per row (TW = 8 when rows are short, 32 otherwise),
// kAnaRowsPerGroup rows per group.  With TW = 8, rows of more than
// kAnaLongK entries are listed and left to a second, warp-wide pass
// (LISTED: the rows are P.longk_rows[0 .. n_longk)).
constexpr int kAnaLongK = 64;

template <int TW, bool LISTED>
__global__ void __launch_bounds__(kAnaThreads) k_analyze(CsrDev A, CsrDev B, PlanDev P)
{
    constexpr int NW = kAnaThreads / 32;
    constexpr int NGR = kAnaThreads / TW;  // groups per block
    constexpr int RPG = LISTED ? 1 : kAnaRowsPerGroup;  // rows per group (one listed long row)
    constexpr int RPB = NGR * RPG;
    __shared__ int s_cnt[kNumBins];
    __shared__ int s_base[kNumBins];
    __shared__ int s_bin[RPB];
    __shared__ int s_idx[RPB];
    __shared__ unsigned long long s_flop[NW];
    __shared__ int s_maxk[NW];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gl = threadIdx.x & (TW - 1);    // lane in the group
    const int grp = threadIdx.x / TW;         // group in the block
    const unsigned gm = TW == 32 ? kFull : (((1u << TW) - 1u) << (lane & ~(TW - 1)));
    if (threadIdx.x < kNumBins)
        s_cnt[threadIdx.x] = 0;
    __syncthreads();
    const int M = A.M, K = B.M;
    const int nrows = LISTED ? P.cnt->n_longk : M;
    const int row0 = blockIdx.x * RPB;
    unsigned long long gflop = 0;
    int gmaxk = 0;
    for (int r = 0; r < RPG; r++) {
        const int slot = grp * RPG + r;
        if (row0 + slot >= nrows) {
            if (gl == 0)
                s_bin[slot] = -1;
            continue;
        }
        const int row = LISTED ? P.longk_rows[row0 + slot] : row0 + slot;
        int a0 = A.rpt[row];
        int a1 = A.rpt[row + 1];
        if (TW < 32 && a1 - a0 > kAnaLongK && a0 >= 0 && a1 <= A.nnz) {
            if (gl == 0) {
                P.longk_rows[atomicAdd(&P.cnt->n_longk, 1)] = row;
                s_bin[slot] = -1;
            }
            continue;
        }
        long long f = 0;
        int nl = 0, leaf = -1;
        bool bad = false;
        if (a0 < 0 || a1 < a0 || a1 > A.nnz) {  // malformed row pointers: treat the row as empty
            bad = true;
            a0 = a1 = 0;
        }
        // UN entries a lane in flight; the listed long rows also take the
        // first and last column of every nonempty list in the same pass (the
        // column range), so their long lists are walked once
        constexpr int UN = LISTED ? 8 : 4;
        int mn = INT_MAX, mx = -1;
        for (int jb = a0 + gl; jb < a1; jb += UN * TW) {
            int b[UN], bs[UN], be[UN];
#pragma unroll
            for (int u = 0; u < UN; u++) {
                const int j = jb + u * TW;
                b[u] = j < a1 ? A.col[j] : -1;
            }
#pragma unroll
            for (int u = 0; u < UN; u++) {
                const int j = jb + u * TW;
                bs[u] = be[u] = 0;
                if (j < a1) {
                    if ((unsigned)b[u] < (unsigned)K) {
                        bs[u] = B.rpt[b[u]];
                        be[u] = B.rpt[b[u] + 1];
                    } else {
                        bad = true;
                    }
                }
            }
            if (LISTED) {
                int c0[UN], c1[UN];
#pragma unroll
                for (int u = 0; u < UN; u++) {
                    c0[u] = INT_MAX;
                    c1[u] = -1;
                    if (be[u] > bs[u]) {
                        c0[u] = B.col[bs[u]];
                        c1[u] = B.col[be[u] - 1];
                    }
                }
#pragma unroll
                for (int u = 0; u < UN; u++) {
                    mn = min(mn, c0[u]);
                    mx = max(mx, c1[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < UN; u++) {
                const int j = jb + u * TW;
                if (j < a1) {
                    const int len = be[u] - bs[u];
                    P.abs[j] = bs[u];
                    P.alen[j] = len;
                    f += len;
                    if (len > 0) {
                        nl++;
                        leaf = max(leaf, j - a0);
                    }
                }
            }
        }
        f = grp_sum<TW>(f, gm);
        nl = grp_sum<TW>(nl, gm);
        leaf = grp_max<TW>(leaf, gm);
        bad = (__ballot_sync(gm, bad) & gm) != 0u;
        const bool ovf = f > INT_MAX;
        if (ovf)
            f = INT_MAX;
        // row class (f, nl, a0, a1 are uniform in the group)
        int bin;
        if (f == 0)
            bin = kBinEmpty;
        else if (nl == 1)
            bin = kBinCopy;
        else if (f <= kWarpMaxFlop)
            bin = kBinWarp;
        else if (f <= kMg2F && a1 - a0 <= kMidMaxK)  // unless the column range is too wide
            bin = f <= kMtF    ? kBinMidTile
                  : f <= kMt2F ? kBinMidTile2
                  : (f <= kMwF && a1 - a0 <= kMwMaxK) ? kBinMidWarp
                  : (f <= kMgF && a1 - a0 <= kMwMaxK) ? kBinMidGroup
                               : kBinMidGroup2;
        else if (f <= P.mid_limit && 2 * nl <= P.mid_limit && a1 - a0 <= kMidMaxK)
            bin = kBinBatch;
        else if (a1 - a0 <= kSegMaxK)
            bin = kBinHeavy;  // segmented (brm_seg.cuh)
        else
            bin = kBinMid;    // row CTA / spill path
        if (bin == kBinHeavy || bin == kBinMidWarp || bin == kBinMidGroup || bin == kBinMidTile ||
            bin == kBinMidTile2 || bin == kBinMidGroup2) {
            // column range of the row for the segment planning and the warp
            // mid rows' keys: the first and last column of every nonempty list
            for (int jb = a0 + gl; !LISTED && jb < a1; jb += 4 * TW) {
                int c0[4], c1[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int j = jb + u * TW;
                    c0[u] = INT_MAX;
                    c1[u] = -1;
                    if (j < a1) {
                        const int len = P.alen[j];
                        if (len > 0) {
                            const int bs = P.abs[j];
                            c0[u] = B.col[bs];
                            c1[u] = B.col[bs + len - 1];
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    mn = min(mn, c0[u]);
                    mx = max(mx, c1[u]);
                }
            }
            mn = grp_min<TW>(mn, gm);
            mx = grp_max<TW>(mx, gm);
            if (gl == 0)
                P.crange[row] = make_int2(mn, mx);
            if ((bin == kBinMidWarp && (long long)mx - mn >= (1ll << kMwRangeBits)) ||
                (bin == kBinMidGroup && (long long)mx - mn >= (1ll << kMgRangeBits)) ||
                ((bin == kBinMidTile || bin == kBinMidTile2) &&
                 (long long)mx - mn >= (1ll << kMtRangeBits)) ||
                (bin == kBinMidGroup2 && (long long)mx - mn >= (1ll << kMg2RangeBits)))
                bin = (f <= P.mid_limit && 2 * nl <= P.mid_limit) ? kBinBatch : kBinHeavy;
            if (bin == kBinHeavy && a1 - a0 > kSegMaxK)
                bin = kBinMid;
        }
        if (gl == 0) {
            if (bad)
                atomicOr(&P.cnt->err, kErrBadInput);
            if (ovf)
                atomicOr(&P.cnt->err, kErrOverflow);
            P.flop[row] = (int)f;
            if (bin == kBinHeavy)
                P.seg_base[row] = atomicAdd(&P.cnt->seg_cap, seg_bound(f, B.N, P.seg_cut));
            P.mid_flop[row] = bin == kBinBatch ? max((int)f, 2 * nl) : 0;  // batch weight
            P.mw_flop[row] =
                (bin == kBinMidWarp || bin == kBinMidGroup || bin == kBinMidTile ||
                 bin == kBinMidTile2 || bin == kBinMidGroup2)
                    ? (int)f
                    : 0;
            P.spill[row] = 0;
            if (bin == kBinEmpty)
                P.nnz[row] = 0;
            else if (bin == kBinCopy) {
                P.nnz[row] = (int)f;
                P.copy_leaf[row] = leaf;
            }
            if (bin == kBinHeavy && f > kHugeFlop) {
                // the planning takes these first, so the longest rows do not
                // start last and finish after every other block
                const int h = atomicAdd(&P.cnt->n_huge, 1);
                if (BRM_IN(P.cnt, M - 1 - h, M))
                    P.rows[(size_t)kBinHeavy * M + (M - 1 - h)] = row;
                bin = -2;
            }
            s_bin[slot] = bin;
            s_idx[slot] = (bin < 0 || bin == kBinEmpty || bin == kBinBatch) ? 0 : atomicAdd(&s_cnt[bin], 1);
            gflop += (unsigned long long)f;
            gmaxk = max(gmaxk, a1 - a0);
        }
    }
    // per warp: the groups' totals (held by their first lanes)
    {
        unsigned long long wf = grp_sum<32>(gflop, kFull);
        int wk = grp_max<32>(gmaxk, kFull);
        if (lane == 0) {
            s_flop[w] = wf;
            s_maxk[w] = wk;
        }
    }
    __syncthreads();
    if (threadIdx.x < kNumBins)
        s_base[threadIdx.x] =
            s_cnt[threadIdx.x] ? atomicAdd(&P.cnt->bin_count[threadIdx.x], s_cnt[threadIdx.x]) : 0;
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        int mk = 0;
        for (int i = 0; i < NW; i++) {
            t += s_flop[i];
            mk = max(mk, s_maxk[i]);
        }
        if (t)
            atomicAdd(&P.cnt->total_flop, t);
        atomicMax(&P.cnt->max_k, mk);
    }
    __syncthreads();
    for (int slot = threadIdx.x; slot < RPB; slot += kAnaThreads) {
        int bin = s_bin[slot];
        if (bin > kBinEmpty && bin != kBinBatch && BRM_IN(P.cnt, s_base[bin] + s_idx[slot], M))
            P.rows[(size_t)bin * M + s_base[bin] + s_idx[slot]] =
                LISTED ? P.longk_rows[row0 + slot] : row0 + slot;
    }
}

void launch_analyze(const CsrDev &A, const CsrDev &B, const PlanDev &P, cudaStream_t s)
{
    if (A.M <= 0)
        return;
    constexpr int RPB32 = (kAnaThreads / 32) * kAnaRowsPerGroup;
    // eight lanes a row when rows average at most 12 entries; the few long
    // rows then go to a warp-wide pass over their list (at most all rows)
    if ((long long)A.nnz <= 12ll * A.M) {
        constexpr int RPB = (kAnaThreads / 8) * kAnaRowsPerGroup;
        k_analyze<8, false><<<(A.M + RPB - 1) / RPB, kAnaThreads, 0, s>>>(A, B, P);
        count_launch();
        const long long most = std::min<long long>(A.M, (long long)A.nnz / (kAnaLongK + 1));
        constexpr int RPBL = kAnaThreads / 32;  // one listed row per warp
        const int g = (int)std::max<long long>(1, (most + RPBL - 1) / RPBL);
        k_analyze<32, true><<<g, kAnaThreads, 0, s>>>(A, B, P);
    } else {
        k_analyze<32, false><<<(A.M + RPB32 - 1) / RPB32, kAnaThreads, 0, s>>>(A, B, P);
    }
    count_launch();
}

// ---------------------------------------------------------------------------
// Exclusive scan (reduce, scan of tile sums, downsweep), out[n] = total.
// Replaces opt_prefix_sum (spgemm.h:179-187) for crpt and scan_floprC.
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int *in, int n,
                                                              long long *tile_sums)
{
    __shared__ long long ws[kScanThreads / 32 + 1];
    const long long base = (long long)blockIdx.x * kScanTile;
    long long s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        long long idx = base + (long long)i * kScanThreads + threadIdx.x;
        if (idx < n)
            s += in[idx];
    }
    long long t = block_sum<kScanThreads>(s, ws);
    if (threadIdx.x == 0)
        tile_sums[blockIdx.x] = t;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(long long *tile_sums, int ntiles)
{
    __shared__ long long ws[kScanThreads / 32 + 1];
    long long carry = 0;
    for (int base = 0; base < ntiles; base += kScanThreads) {
        int idx = base + threadIdx.x;
        long long v = idx < ntiles ? tile_sums[idx] : 0;
        long long tot;
        long long ex = block_excl_scan<kScanThreads>(v, ws, &tot);
        if (idx < ntiles)
            tile_sums[idx] = carry + ex;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0)
        tile_sums[ntiles] = carry;
}

template <typename OutT>
__global__ void __launch_bounds__(kScanThreads) k_scan_down(const int *in, int n,
                                                            const long long *tile_sums,
                                                            OutT *out, Counters *cnt)
{
    __shared__ long long ws[kScanThreads / 32 + 1];
    const long long base = (long long)blockIdx.x * kScanTile;
    // blocked arrangement: thread t owns items [t*I, t*I+I) of the tile
    long long v[kScanItems];
    long long s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        long long idx = base + (long long)threadIdx.x * kScanItems + i;
        v[i] = idx < n ? in[idx] : 0;
        s += v[i];
    }
    long long tot;
    long long ex = block_excl_scan<kScanThreads>(s, ws, &tot);
    long long run = tile_sums[blockIdx.x] + ex;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        long long idx = base + (long long)threadIdx.x * kScanItems + i;
        if (idx < n) {
            if (sizeof(OutT) == 4 && run > INT_MAX) {
                if (cnt)
                    atomicOr(&cnt->err, kErrOverflow);
                out[idx] = (OutT)INT_MAX;
            } else {
                out[idx] = (OutT)run;
            }
        }
        run += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        long long total = tile_sums[gridDim.x];
        if (cnt)
            cnt->cnnz = total;
        if (sizeof(OutT) == 4 && total > INT_MAX) {
            if (cnt)
                atomicOr(&cnt->err, kErrOverflow);
            out[n] = (OutT)INT_MAX;
        } else {
            out[n] = (OutT)total;
        }
    }
}

size_t scan_tmp_bytes(int n)
{
    size_t tiles = (size_t)(n + kScanTile - 1) / kScanTile;
    return (tiles + 2) * sizeof(long long);
}

template <typename OutT>
static void scan_impl(const int *in, OutT *out, int n, Counters *cnt, void *tmp, cudaStream_t s)
{
    long long *ts = (long long *)tmp;
    int tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 0)
        tiles = 1;
    k_scan_reduce<<<tiles, kScanThreads, 0, s>>>(in, n, ts);
    count_launch();
    k_scan_tiles<<<1, kScanThreads, 0, s>>>(ts, tiles);
    count_launch();
    k_scan_down<OutT><<<tiles, kScanThreads, 0, s>>>(in, n, ts, out, cnt);
    count_launch();
}

void launch_scan_i32(const int *in, int *out, int n, Counters *cnt, void *tmp, cudaStream_t s)
{
    scan_impl<int>(in, out, n, cnt, tmp, s);
}

void launch_scan_i64(const int *in, long long *out, int n, void *tmp, cudaStream_t s)
{
    scan_impl<long long>(in, out, n, nullptr, tmp, s);
}

// ---------------------------------------------------------------------------
// Upper compaction (spgemm.h:429-444): one warp per row, C_bar -> C.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_compact(int M, const long long *scan_flop, const int *len,
                                                 const int *bar_col, const T *bar_val,
                                                 const int *crpt, int *ccol, T *cval, Counters *cnt)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int row = gw; row < M; row += nw) {
        const long long src = scan_flop[row];
        const int dst = crpt[row];
        int n = len[row];
        if (n > 0 && !(BRM_IN(cnt, (long long)dst + n - 1, crpt[M]) &&
                       BRM_IN(cnt, src + n - 1, (long long)cnt->total_flop)))
            n = 0;  // checked build: a row outside C or C_bar is skipped
        for (int q = lane; q < n; q += 32) {
            ccol[dst + q] = bar_col[src + q];
            cval[dst + q] = bar_val[src + q];
        }
    }
}

void launch_compact(int dtype, const PlanDev &P, const int *bar_col, const void *bar_val,
                    const int *crpt, int *ccol, void *cval, cudaStream_t s)
{
    if (P.M <= 0)
        return;
    int grid = (P.M + 7) / 8;
    if (grid > 65535 * 4)
        grid = 65535 * 4;
    if (dtype == 0) {
        k_compact<double><<<grid, 256, 0, s>>>(P.M, P.scan_flop, P.nnz, bar_col,
                                                (const double *)bar_val, crpt, ccol, (double *)cval,
                                                P.cnt);
        count_launch();
    } else {
        k_compact<float><<<grid, 256, 0, s>>>(P.M, P.scan_flop, P.nnz, bar_col,
                                               (const float *)bar_val, crpt, ccol, (float *)cval,
                                               P.cnt);
        count_launch();
    }
}

// ---------------------------------------------------------------------------
// CSR validation (the invariants the reference's reader enforces,
// CSR.cpp:454-477): rpt[0] == 0, rpt non-decreasing, rpt[M] == nnz, columns in
// [0, ncols) and strictly increasing within each row.  One warp per row;
// *bad_row receives the smallest offending row (atomicMin), -1 if none was
// seen (the host initialises it to INT_MAX).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_validate(CsrDev X, int ncols, int *bad_row)
{
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    if (gw == 0 && lane == 0) {
        if (X.rpt[0] != 0)
            atomicMin(bad_row, 0);
        if (X.rpt[X.M] != X.nnz)
            atomicMin(bad_row, X.M > 0 ? X.M - 1 : 0);
    }
    for (int row = gw; row < X.M; row += nw) {
        const int s = X.rpt[row], e = X.rpt[row + 1];
        bool bad = (s > e) || (s < 0) || (e > X.nnz);
        if (!bad) {
            for (int j = s + lane; j < e; j += 32) {
                int c = X.col[j];
                if ((unsigned)c >= (unsigned)ncols)
                    bad = true;
                else if (j + 1 < e && X.col[j + 1] <= c)
                    bad = true;
            }
        }
        if (__any_sync(kFull, bad) && lane == 0)
            atomicMin(bad_row, row);
    }
}

void launch_validate(const CsrDev &X, int ncols, int *bad_row, cudaStream_t s)
{
    int grid = (X.M + 7) / 8;
    if (grid < 1)
        grid = 1;
    if (grid > 65535 * 4)
        grid = 65535 * 4;
    k_validate<<<grid, 256, 0, s>>>(X, ncols, bad_row);
    count_launch();
}

}  // namespace brm

namespace brm {

__global__ void k_pipe_admit(PlanDev P, int M, PipeCaps caps, int stage)
{
    Counters *c = P.cnt;
    bool bad;
    if (stage == 0)
        bad = (long long)c->total_flop > caps.products || (long long)c->seg_cap > caps.seg_slots ||
              P.mid_pre[M] + P.mw_pre[M] > caps.products;
    else
        bad = (long long)c->table_cap > caps.table || (long long)c->spill_bytes > caps.spill_bytes;
    if (bad) {
        c->abort = 1;
        atomicOr(&c->err, kErrCapacity);
    }
}

void launch_pipe_admit(const PlanDev &P, int M, const PipeCaps &caps, int stage, cudaStream_t s)
{
    k_pipe_admit<<<1, 1, 0, s>>>(P, M, caps, stage);
    count_launch();
}

}  // namespace brm

// SM version of the device code this library runs on the current device.
extern "C" int brm_device_code_version(int *sm)
{
    if (!sm)
        return BRM_ERR_INVALID_VALUE;
    cudaFuncAttributes fa;
    const cudaError_t e = cudaFuncGetAttributes(&fa, brm::k_scan_reduce);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return e == cudaErrorNoDevice ? BRM_ERR_NO_DEVICE : BRM_ERR_CUDA;
    }
    *sm = fa.binaryVersion;
    return BRM_SUCCESS;
}
