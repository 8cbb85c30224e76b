// brm_plan.h -- data shared between the host orchestration and the kernels.
//
// A plan is the device state that the symbolic phase leaves for the numeric
// phase (the reference keeps the same state in local arrays between its
// symbolic and numeric loops, BRMerge-SpGEMM/inc/spgemm.h:476-578).
#pragma once

#include <cstdint>

#include <vector_types.h>

namespace brm {

// Tuning constants of the row kernels.
constexpr int kRowThreads = 512;            // threads of a row CTA
constexpr int kCap = 6144;                  // products staged in shared memory per window
constexpr int kLMax = 4096;                 // lists (A-row entries) kept in shared memory
constexpr int kChunkWords = 4096;           // bitmap words per column chunk
constexpr int kChunkBits = kChunkWords * 32;  // columns per chunk (131072)
constexpr int kWarpMaxFlop = 32;            // rows up to this many products go to warp kernels
constexpr int kHeavyFlop = 4 * kCap;        // rows above this are scheduled first
constexpr int kRadixBits = 7;

// Batched mid-row kernels: rows with more than kWarpMaxFlop products, weight
// w = max(products, 2 * nonempty lists) <= kMidFlop and at most kMidMaxK A
// entries are packed, in row order, into batches (a batch starts where the
// row-order prefix of w crosses a multiple of kMidFlop, so a batch holds at
// most kMidCap products and kMidMaxLists nonempty lists).
constexpr int kMidThreads = 256;
constexpr int kMidCap = 4096;
constexpr int kMidFlop = kMidCap / 2;
constexpr int kMidMaxLists = kMidCap / 2;
constexpr int kMidMaxK = 255;
constexpr int kMidMaxRows = kMidCap / (kWarpMaxFlop + 1) + 2;

// Warp mid rows: more than kWarpMaxFlop and at most kMwF products, at most
// kMwMaxK A entries, columns within a range below 2^kMwRangeBits; one warp
// each.  Group rows: up to kMgF products and kMwMaxK A entries, range below
// 2^kMgRangeBits, four warps each; longer group rows (up to kMg2F products,
// kMidMaxK A entries) in their own class.  All take precedence over the
// batched mid rows and over the segmented heavy rows.  Holding the first two
// classes to 64 lists keeps their merge-tree stacks at seven levels and
// their kernels within 80 registers without spills.
constexpr int kMwF = 768;
constexpr int kMwMaxK = 64;
constexpr int kMwRangeBits = 22;
constexpr int kMtF = 64;          // tile rows: at most 64 products, half a warp each
constexpr int kMt2F = 128;        // second tile class: at most 128 products
constexpr int kMtRangeBits = 25;
constexpr int kMgF = 3072;
constexpr int kMgRangeBits = 20;
constexpr int kMg2F = 5888;       // second group class: two groups a CTA fit 2 CTAs an SM
constexpr int kMg2RangeBits = 19;
// Subsets of the mid-row kernels (they can run on different streams).
constexpr int kMidGroups = 1;     // the batched mid rows and the four-warp group rows
constexpr int kMidWarps = 2;      // the warp and tile rows

// Segmented heavy rows: a row that is not a mid row is cut, at 32-column word
// (or, inside very dense words, column) boundaries, into column segments of at
// most kSegCap products within one planning chunk of kPlanBits columns.  The
// planning pass records, for every segment boundary and every list of the
// row, where the list crosses the boundary (the split table), so each segment
// is an independent unit of work.
#ifndef BRM_SEG_THREADS
#define BRM_SEG_THREADS 256
#endif
#ifndef BRM_SEG_CAP
#define BRM_SEG_CAP 3072
#endif
constexpr int kSegThreads = BRM_SEG_THREADS;
constexpr int kSegCap = BRM_SEG_CAP;
// Target products between cuts (a runtime knob, brm_tuning.seg_cut): the
// default and the largest accepted.  Segments average about the target, so a
// larger one means fewer segments (less fixed work per product in the
// segment kernel, a smaller split table) but more dense planning groups
// (above kSegCap - target products), whose columns are counted one by one.
// R-MAT n=2^18 C = A*A one-call Precise: 1536 -> 3.10 ms, 2048 -> 3.02,
// 2304 -> 2.94, 2560 -> 3.11, 2688 -> 3.11 (same output).
constexpr int kSegCut = kSegCap * 3 / 4;
constexpr int kSegMaxCut = kSegCap * 7 / 8;
constexpr int kSegMaxK = 65535;           // leaf index stored in 16 bits
constexpr int kHugeFlop = 16 * kSegCap;   // heavy rows planned first (longest first)
constexpr int kMaxParts = 16;             // row parts of a numeric phase run part by part
constexpr int kPlanWordsLog2 = 13;
constexpr int kPlanWords = 1 << kPlanWordsLog2;  // bitmap words per planning chunk
constexpr int kPlanBits = kPlanWords * 32;       // 2^18 columns
constexpr int kSumWords = kPlanBits / 1024;      // summary words of a segment bitmap

// Device error bits, OR-ed into Counters::err and read back by the host.
enum DevErr : int {
    kErrNone = 0,
    kErrWindowOverflow = 1,  // a numeric window exceeded its shared-memory capacity
    kErrNnzMismatch = 2,     // numeric row length differs from the symbolic count
    kErrSpillCapacity = 4,   // spill scratch smaller than a spill row needs
    kErrOverflow = 8,        // an int32 quantity overflowed
    kErrBadInput = 16,       // an index out of range seen by a kernel
    kErrCapacity = 32,       // a batch exceeded a captured pipeline's capacities
    kErrChecked = 64,        // a bounds check of the checked build failed (brm_check.cuh)
};

// Row classes assigned by the analysis kernel.
enum RowBin : int {
    kBinEmpty = 0,  // no products: nnz 0
    kBinCopy = 1,   // exactly one nonempty list: C row = a * B row
    kBinWarp = 2,   // <= kWarpMaxFlop products, >= 2 nonempty lists
    kBinHeavy = 3,  // row CTA, scheduled first
    kBinMid = 4,    // row CTA
    kBinBatch = 5,  // batched mid-row kernels (no row list: row-order batches)
    kBinMidWarp = 6,  // one warp per row (brm_midwarp.cuh)
    kBinMidGroup = 7, // four warps per row (brm_midwarp.cuh)
    kBinMidTile = 8,  // half a warp per row, products sorted in registers (brm_midwarp.cuh)
    kBinMidTile2 = 9, // the same with twice the products
    kBinMidGroup2 = 10,  // four warps per row, longer rows (brm_midwarp.cuh)
    kNumBins = 11,
};

// Device counters (one struct in device memory, zeroed per phase).
struct Counters {
    int bin_count[kNumBins];
    int spill_count;
    int work_sym;      // dynamic row counter of the symbolic row kernel
    int work_num;      // dynamic row counter of the numeric row kernel
    int err;           // OR of DevErr bits
    int max_k;         // longest A row
    unsigned long long total_flop;
    unsigned long long spill_bytes;  // scratch reserved for spill rows
    long long cnnz;    // total nnz of C (int64 before the int32 check)
    int n_batch;       // number of mid-row batches
    int work_bsym;     // dynamic batch counter, symbolic
    int work_bnum;     // dynamic batch counter, numeric
    int work_seg;      // dynamic segment counter, numeric
    unsigned long long seg_cap;    // descriptor slots reserved by the analysis
    unsigned long long table_cap;  // split-table entries reserved by the planning
    int n_seg;         // segments written by the planning
    int work_plan;     // dynamic row counter of the heavy-row planning
    int n_huge;        // heavy rows above kHugeFlop products (listed from the end)
    int n_longk;       // rows the narrow analysis left to the warp-wide pass
    // long columns of the segment kernel handed to the column reducers:
    // columns and elements reserved so far (two counters, so neither can
    // overflow into the other however many columns a call has)
    unsigned long long long_cols;
    unsigned long long long_elems;
    // set by the capacity checks of a captured batch pipeline when the batch
    // does not fit its buffers; every kernel that writes at data-dependent
    // offsets then returns at once (the call reports BRM_ERR_CAPACITY)
    int abort;
    // first failed bounds check of the checked build: source line, index, bound
    int chk_line;
    long long chk_idx;
    long long chk_bound;
    // dynamic row counters of the warp / four-warp mid-row kernels (one per
    // shape) and the groups of a launch that have finished; the last group
    // of a launch sets both back to zero, so every launch starts from zero
    // whatever phase or pipeline runs it
    int work_mw[3];
    int done_mw[3];
};

// Descriptor slots reserved for a heavy row with F products and the cut
// target `cut`: the cut rule makes at most F / cut cuts at product
// thresholds (plus one per chunk), 2 per dense group (a group with more than
// dense = kSegCap - cut products; at most F / dense of them) and at most
// 2 h / cut + 1 inside a dense group of h products, plus one chunk start per
// kPlanBits columns: at most 3 F / cut + 3 F / dense <= 6 F / min(cut, dense)
// and the chunk terms.
__host__ __device__ inline unsigned long long seg_bound(long long F, int N, int cut)
{
    const int m = cut < kSegCap - cut ? cut : kSegCap - cut;
    return 6ull * (unsigned long long)((F + m - 1) / m) +
           2ull * ((unsigned)N / (unsigned)kPlanBits) + 8ull;
}

// Runtime policy knobs of the row classes (chosen by brm_autotune or
// brm_set_tuning; every capacity stays compile-time): the heavy-row cut
// target seg_cut in [kMinSegCut, kSegMaxCut] (segments hold at most kSegCap
// products whatever the target) and the mid-row weight limit mid_flop in
// [kMinMidFlop, kMidFlop] (batches hold at most 2 * mid_flop <= kMidCap).
// The results do not depend on them: only where rows and segments are cut.
constexpr int kMinSegCut = 256;
constexpr int kMinMidFlop = 128;

// One column segment of a heavy row.
struct SegDesc {
    int row;
    int c_lo;       // first column of the segment
    int c_hi;       // one past the last column
    int u_off;      // distinct columns of the row before c_lo
    int bidx;       // boundary index of c_lo in the row's split table
    int nprod;      // products in the segment
    long long tab;  // split-table offset of the row (boundary-major, k entries each)
};

// A segment as the segment kernel reads it: one 48-byte record per entry of
// the segment list (in list order), written by k_split, so that a segment
// needs a single dependent load after the work counter (and the next one is
// copied into shared memory while the current segment runs).
struct __align__(16) SegRun {
    long long sp;  // split-table offset of the segment's first boundary row (tab + bidx * k)
    int row;
    int c_lo;
    int c_hi;
    int u_off;     // distinct columns of the row before c_lo
    int nprod;
    int a0;        // A row start and length
    int k;
    int next_u;    // distinct columns of the row before the next segment (or its nnz)
};
static_assert(sizeof(SegRun) == 48, "three 16-byte copies");

// A column of a heavy-row segment with many products, handed from the
// segment kernel to the column reducer: its products' leaves and values in
// leaf order at [off, off + len) of the long-column scratch, and the output
// position.  len < 0: the segment kernel reduced the column itself.
struct LongCol {
    long long out;  // index into (ccol, cval)
    long long off;  // first element in the scratch
    int col;        // column of C
    int len;
};

// Device arrays of a plan (all sized for M rows unless noted).
struct PlanDev {
    int M;
    int *flop;        // [M] products per row
    int *nnz;         // [M] symbolic row length (Upper: numeric row length)
    int *rows;        // [kNumBins * M] row lists, bin b at rows + b*M
    int *copy_leaf;   // [M] leaf of the single nonempty list (copy rows)
    unsigned char *spill;  // [M] 1 if the row takes the spill path
    int *spill_rows;  // [M] spill row list
    unsigned long long *spill_off;  // [M] scratch byte offset per spill list entry
    long long *scan_flop;  // [M+1] exclusive scan of flop (Upper)
    int *abs;              // [nnz(A)] start of B row acol[j] (list start of A entry j)
    int *alen;             // [nnz(A)] length of B row acol[j] (0 if acol[j] is out of range)
    int *mid_flop;         // [M] products of batched mid rows, 0 for other rows
    long long *mid_pre;    // [M+1] exclusive scan of mid_flop
    int *mw_flop;          // [M] products of warp mid rows, 0 for other rows
    long long *mw_pre;     // [M+1] exclusive scan of mw_flop (one-call scratch after mid_pre[M])
    int *longk_rows;       // [M] rows with many A entries, analysed by whole warps
    int *batch_start;      // [M+1] first row of each mid batch
    unsigned long long *seg_base;  // [M] first descriptor slot of each heavy row
    int *seg_n;            // [M] segments of each heavy row (0: not segmented)
    int2 *crange;          // [M] smallest and largest column of each heavy row (x > y: none)
    SegDesc *seg;          // [Counters::seg_cap] segment descriptors (numbered per row)
    int *seg_list;         // [Counters::seg_cap] descriptor slot of every written segment
    SegRun *run;           // [Counters::seg_cap] records of the segment list (numeric phase)
    int *split;            // [Counters::table_cap] split table (numeric phase)
    LongCol *long_col;     // [long_cap_cols] long-column descriptors (numeric phase)
    unsigned short *long_leaf;  // [long_cap_elems] leaves of the long columns' products
    void *long_val;        // [long_cap_elems] their values (the value type)
    long long long_cap_cols;
    long long long_cap_elems;
    // numeric launches may cover only rows [r_lo, r_hi) (a part of C copied
    // back while the next part computes); seg_range (device, 2 ints), when
    // set, is the part's range of seg_list
    int r_lo;
    int r_hi;
    const int *seg_range;
    // policy knobs (see kMinSegCut): heavy-row cut target, mid-row weight limit
    int seg_cut;
    int mid_limit;
    // entries of the arrays the numeric kernels write (C, or C_bar for
    // Upper) and of the one-call mid-row scratch; the bounds of the checked
    // build
    long long c_cap;
    long long mid_cap;
    Counters *cnt;
    // host side only: the launches the plan needs (kLive* bits); all ones
    // when the host does not know the class counts (a captured pipeline)
    unsigned live;
};

// Launch mask of a plan (PlanDev::live): bit b set when row class b (RowBin)
// has rows, kLiveSegs when heavy rows were cut into segments.  The launchers
// skip the kernels of empty classes, which for small products are most of
// the launches of a call.
constexpr unsigned kLiveSegs = 1u << 30;
constexpr unsigned kLiveAll = 0xffffffffu;
constexpr unsigned live_bit(int bin) { return 1u << bin; }
constexpr unsigned kLiveMidRows = live_bit(kBinBatch) | live_bit(kBinMidWarp) |
                                  live_bit(kBinMidGroup) | live_bit(kBinMidTile) |
                                  live_bit(kBinMidTile2) | live_bit(kBinMidGroup2);
inline bool plan_live(const PlanDev &P, unsigned bits) { return (P.live & bits) != 0; }

// Capacities of a captured batch pipeline: every buffer sized by a count the
// planning computes on the device is grown to these once, and admission
// kernels compare each batch's counts with them (Counters::abort).
struct PipeCaps {
    long long rows;         // rows of the stacked A (and of C)
    long long nnz_a;        // entries of the stacked A
    long long b_rows;       // rows of the stacked B
    long long nnz_b;        // entries of the stacked B
    long long cols;         // columns of the stacked B
    long long products;     // intermediate products (bounds nnz(C) and the mid-row scratch)
    long long seg_slots;    // heavy-row segment descriptors
    long long table;        // split-table entries
    long long spill_bytes;  // spill scratch
};

struct CsrDev {
    int M, N, nnz;
    const int *rpt;
    const int *col;
    const void *val;
};

}  // namespace brm
