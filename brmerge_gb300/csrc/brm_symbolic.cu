// brm_symbolic.cu -- symbolic phase launchers (exact row nnz, spill routing).
#include "brm_kernels.h"
#include "brm_mid.cuh"
#include "brm_midwarp.cuh"
#include "brm_rows.cuh"
#include "brm_seg.cuh"

namespace brm {

void launch_batches(const PlanDev &P, int M, void *tmp, cudaStream_t s)
{
    if (M <= 0)
        return;
    launch_scan_i64(P.mid_flop, P.mid_pre, M, tmp, s);
    launch_scan_i64(P.mw_flop, P.mw_pre, M, tmp, s);
    k_batch_starts<0><<<(M + 1 + 255) / 256, 256, 0, s>>>(P, M);
    count_launch();
}

void launch_symbolic(const CsrDev &A, const CsrDev &B, const PlanDev &P, int num_sms,
                     bool only_heavy, bool skip_mid, cudaStream_t s)
{
    if (A.M <= 0)
        return;
    if (!only_heavy) {
        if (plan_live(P, live_bit(kBinWarp))) {
            k_warp_symbolic<0><<<num_sms * 8, 256, 0, s>>>(A, B, P);
            count_launch();
        }
        if (!skip_mid) {
            if (plan_live(P, live_bit(kBinBatch))) {
                const size_t msm = MidSymLayout::bytes;
                cudaFuncSetAttribute(k_mid_symbolic<0>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msm);
                k_mid_symbolic<0><<<num_sms * 2, kMidThreads, msm, s>>>(A, B, P);
                count_launch();
            }
            launch_mid_warp<double, kMwSymbolic>(A, B, P, nullptr, nullptr, nullptr, num_sms, s);
        }
    }
    // heavy rows: exact nnz and segment plan (both Precise and Upper)
    if (plan_live(P, live_bit(kBinHeavy))) {
        const size_t psm = PlanLayout::bytes;
        cudaFuncSetAttribute(k_heavy_plan<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)psm);
        k_heavy_plan<0><<<num_sms * 3, kPlanThreads, psm, s>>>(A, B, P);
        count_launch();
    }
    if (!plan_live(P, live_bit(kBinMid)))
        return;
    const size_t smem = SymLayout::bytes;
    if (only_heavy) {
        cudaFuncSetAttribute(k_rows_symbolic<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        k_rows_symbolic<true><<<num_sms * 4, kRowThreads, smem, s>>>(A, B, P);
        count_launch();
    } else {
        cudaFuncSetAttribute(k_rows_symbolic<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        k_rows_symbolic<false><<<num_sms * 4, kRowThreads, smem, s>>>(A, B, P);
        count_launch();
    }
}

void launch_seg_partition(const PlanDev &P, const int *pb, int nparts, int *cnt, int *fill,
                          int *out, int *ranges, int num_sms, cudaStream_t s)
{
    k_seg_part_count<0><<<num_sms * 4, 256, 0, s>>>(P, pb, nparts, cnt);
    count_launch();
    k_seg_part_scatter<0><<<num_sms * 4, 256, 0, s>>>(P, pb, nparts, cnt, fill, out, ranges);
    count_launch();
}

}  // namespace brm
