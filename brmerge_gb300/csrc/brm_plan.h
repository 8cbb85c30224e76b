// brm_plan.h -- data shared between the host orchestration and the kernels.
//
// A plan is the device state that the symbolic phase leaves for the numeric
// phase (the reference keeps the same state in local arrays between its
// symbolic and numeric loops, BRMerge-SpGEMM/inc/spgemm.h:476-578).
#pragma once

#include <cstdint>

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

// Device error bits, OR-ed into Counters::err and read back by the host.
enum DevErr : int {
    kErrNone = 0,
    kErrWindowOverflow = 1,  // a numeric window exceeded its shared-memory capacity
    kErrNnzMismatch = 2,     // numeric row length differs from the symbolic count
    kErrSpillCapacity = 4,   // spill scratch smaller than a spill row needs
    kErrOverflow = 8,        // an int32 quantity overflowed
    kErrBadInput = 16,       // an index out of range seen by a kernel
};

// Row classes assigned by the analysis kernel.
enum RowBin : int {
    kBinEmpty = 0,  // no products: nnz 0
    kBinCopy = 1,   // exactly one nonempty list: C row = a * B row
    kBinWarp = 2,   // <= kWarpMaxFlop products, >= 2 nonempty lists
    kBinHeavy = 3,  // row CTA, scheduled first
    kBinMid = 4,    // row CTA
    kNumBins = 5,
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
    int pad[4];
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
    Counters *cnt;
};

struct CsrDev {
    int M, N, nnz;
    const int *rpt;
    const int *col;
    const void *val;
};

}  // namespace brm
