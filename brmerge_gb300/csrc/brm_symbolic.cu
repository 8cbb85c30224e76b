// brm_symbolic.cu -- symbolic phase launchers (exact row nnz, spill routing).
#include "brm_kernels.h"
#include "brm_rows.cuh"

namespace brm {

void launch_symbolic(const CsrDev &A, const CsrDev &B, const PlanDev &P, int num_sms,
                     bool only_heavy, cudaStream_t s)
{
    if (A.M <= 0)
        return;
    if (!only_heavy)
        k_warp_symbolic<0><<<num_sms * 8, 256, 0, s>>>(A, B, P);
    const size_t smem = SymLayout::bytes;
    if (only_heavy) {
        cudaFuncSetAttribute(k_rows_symbolic<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        k_rows_symbolic<true><<<num_sms * 4, kRowThreads, smem, s>>>(A, B, P);
    } else {
        cudaFuncSetAttribute(k_rows_symbolic<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        k_rows_symbolic<false><<<num_sms * 4, kRowThreads, smem, s>>>(A, B, P);
    }
}

}  // namespace brm
