// brm_numeric.cuh -- numeric phase launchers, templated on the value type
// (instantiated once per type in brm_numeric_f64.cu and brm_numeric_f32.cu,
// two translation units that compile in parallel).
#pragma once

#include "brm_kernels.h"
#include "brm_mid.cuh"
#include "brm_midwarp.cuh"
#include "brm_seg.cuh"
#include "brm_rows.cuh"

namespace brm {

template <typename T, bool UPPER>
void numeric_phase(const CsrDev &A, const CsrDev &B, const PlanDev &P, const int *crpt,
                       int *ccol, T *cval, void *spill_scratch, unsigned long long spill_bytes,
                       const int *mid_col, const void *mid_val, int num_sms, cudaStream_t s0,
                       const Fork &fk)
{
    // copy, warp and mid rows on the aux stream (when there is one), beside
    // the split table and the segments of the heavy rows on s0
    cudaStream_t s = s0;
    if (fk.aux) {
        cudaEventRecord(fk.fork, s0);
        cudaStreamWaitEvent(fk.aux, fk.fork, 0);
        s = fk.aux;
    }
    // (kernels of row classes without rows are not launched)
    if (plan_live(P, live_bit(kBinCopy))) {
        k_copy_numeric<T, UPPER><<<num_sms * 8, 256, 0, s>>>(A, B, P, crpt, ccol, cval);
        count_launch();
    }
    if (plan_live(P, live_bit(kBinWarp))) {
        k_warp_numeric<T, UPPER><<<num_sms * 8, 256, 0, s>>>(A, B, P, crpt, ccol, cval);
        count_launch();
    }
    // The mid rows computed with the plan (one-call Precise) are moved into
    // C by a bandwidth-bound copy.  With heavy-row segments it waits for the
    // segment kernel (which holds every SM's registers) and runs beside the
    // latency-bound column reducers that follow it (R-MAT n=2^18 one-call
    // Precise 2.875 -> 2.838 ms; the two reducers on separate streams as
    // well: 2.917 ms).  A numeric phase run in row parts (the host drop-in
    // copies each part back while the next computes) keeps it first.
    const bool compact = mid_col && plan_live(P, kLiveMidRows);
    const bool compact_late = compact && fk.aux && plan_live(P, kLiveSegs) && !P.seg_range;
    if (mid_col) {
        if (compact && !compact_late) {
            k_mid_compact<T><<<num_sms * 8, 256, 0, s>>>(P, A.M, mid_col, (const T *)mid_val,
                                                              crpt, ccol, cval);
            count_launch();
        }
    } else {
        launch_mid_warp<T, UPPER ? kMwUpper : kMwPrecise>(A, B, P, crpt, ccol, cval, num_sms,
                                                          s);
        if (plan_live(P, live_bit(kBinBatch))) {
            const size_t msm = MidNumLayout<T>::bytes;
            cudaFuncSetAttribute(k_mid_numeric<T, UPPER>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msm);
            k_mid_numeric<T, UPPER><<<num_sms * 2, kMidThreads, msm, s>>>(A, B, P, crpt, ccol,
                                                                                cval);
            count_launch();
        }
    }
    if (fk.aux && !compact_late)
        cudaEventRecord(fk.join, fk.aux);
    s = s0;
    if (plan_live(P, kLiveSegs)) {
        k_split<0><<<num_sms * 8, 256, 0, s>>>(A, B, P);
        count_launch();
        const size_t ssm = SegLayout<T>::bytes;
        cudaFuncSetAttribute(k_seg_numeric<T, UPPER>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm);
        // as many segment CTAs as fit on every SM (shared memory and registers)
        static int seg_per_sm = 0;
        if (seg_per_sm <= 0) {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&seg_per_sm,
                                                              k_seg_numeric<T, UPPER>,
                                                              kSegThreads, ssm) != cudaSuccess ||
                seg_per_sm <= 0)
                seg_per_sm = 1;
        }
        k_seg_numeric<T, UPPER><<<num_sms * seg_per_sm, kSegThreads, ssm, s>>>(A, B, P, crpt,
                                                                                ccol, cval);
        count_launch();
        if (compact_late) {
            // fork again after the segments (the event is re-recorded: the
            // aux stream's first wait has already taken its earlier state)
            cudaEventRecord(fk.fork, s0);
            cudaStreamWaitEvent(fk.aux, fk.fork, 0);
            k_mid_compact<T><<<num_sms * 8, 256, 0, fk.aux>>>(P, A.M, mid_col,
                                                                (const T *)mid_val, crpt, ccol,
                                                                cval);
            count_launch();
            cudaEventRecord(fk.join, fk.aux);
        }
        k_long_reduce<T><<<num_sms * 4, 128, 0, s>>>(P, ccol, cval);
        count_launch();
        k_long_warp<T><<<num_sms * 4, 128, 0, s>>>(P, ccol, cval);
        count_launch();
    }
    if (plan_live(P, live_bit(kBinMid))) {
        const size_t smem = NumLayout<T>::bytes;
        cudaFuncSetAttribute(k_rows_numeric<T, UPPER>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_rows_numeric<T, UPPER><<<num_sms, kRowThreads, smem, s>>>(A, B, P, crpt, ccol, cval);
        count_launch();
    }
    if (spill_bytes) {
        k_spill_numeric<T, UPPER><<<num_sms * 4, 32, 0, s>>>(
            A, B, P, crpt, ccol, cval, (unsigned char *)spill_scratch, spill_bytes);
        count_launch();
    }
    if (fk.aux)
        cudaStreamWaitEvent(s0, fk.join, 0);
}

template <typename T>
void launch_numeric_t(bool upper, const CsrDev &A, const CsrDev &B, const PlanDev &P,
                       const int *crpt, int *ccol, void *cval, void *spill_scratch,
                       unsigned long long spill_bytes, const int *mid_col, const void *mid_val,
                       int num_sms, cudaStream_t s, const Fork &fk)
{
    if (A.M <= 0)
        return;
    if (upper)
        numeric_phase<T, true>(A, B, P, crpt, ccol, (T *)cval, spill_scratch, spill_bytes, nullptr,
                          nullptr, num_sms, s, fk);
    else
        numeric_phase<T, false>(A, B, P, crpt, ccol, (T *)cval, spill_scratch, spill_bytes, mid_col,
                           mid_val, num_sms, s, fk);
}

template <typename T>
void launch_mid_scratch_t(const CsrDev &A, const CsrDev &B, const PlanDev &P, int *mid_col,
                            void *mid_val, int num_sms, cudaStream_t s, int which)
{
    if (A.M <= 0)
        return;
    if ((which & kMidGroups) && plan_live(P, live_bit(kBinBatch))) {
        const size_t msm = MidNumLayout<T>::bytes;
        cudaFuncSetAttribute(k_mid_numeric<T, false, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msm);
        k_mid_numeric<T, false, true><<<num_sms * 2, kMidThreads, msm, s>>>(
            A, B, P, nullptr, mid_col, (T *)mid_val);
        count_launch();
    }
    launch_mid_warp<T, kMwScratch>(A, B, P, nullptr, mid_col, (T *)mid_val, num_sms, s, which);
}

}  // namespace brm
