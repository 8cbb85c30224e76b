// brm_numeric_f64.cu -- numeric phase launchers for double values.
#include "brm_numeric.cuh"

namespace brm {

void launch_numeric_f64(bool upper, const CsrDev &A, const CsrDev &B, const PlanDev &P,
                       const int *crpt, int *ccol, void *cval, void *spill_scratch,
                       unsigned long long spill_bytes, const int *mid_col, const void *mid_val,
                       int num_sms, cudaStream_t s, const Fork &fk)
{
    launch_numeric_t<double>(upper, A, B, P, crpt, ccol, cval, spill_scratch, spill_bytes, mid_col,
                          mid_val, num_sms, s, fk);
}

void launch_mid_scratch_f64(const CsrDev &A, const CsrDev &B, const PlanDev &P, int *mid_col,
                            void *mid_val, int num_sms, cudaStream_t s, int which)
{
    launch_mid_scratch_t<double>(A, B, P, mid_col, mid_val, num_sms, s, which);
}

}  // namespace brm
