// C entry points around the reference's own brmerge_precise / brmerge_upper
// (BRMerge-SpGEMM/inc/spgemm.h:468-471, :220-223), compiled from the reference
// sources in place by oracle/build_ref.sh.  Test infrastructure: used to pin
// the oracle restatement and to time the reference on the host cores.
#include "spgemm.h"

extern "C" {

int ref_precise_f64(const int *arpt, const int *acol, const double *aval, const int *brpt,
                    const int *bcol, const double *bval, int M, int K, int N, int **crpt,
                    int **ccol, double **cval, int *cnnz, int nthreads, double *seconds)
{
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
    Precise_Timing t;
    double t0 = omp_get_wtime();
    brmerge_precise(const_cast<int *>(arpt), const_cast<int *>(acol), const_cast<double *>(aval),
                    const_cast<int *>(brpt), const_cast<int *>(bcol), const_cast<double *>(bval),
                    crpt, ccol, cval, M, K, N, cnnz, t);
    if (seconds)
        *seconds = omp_get_wtime() - t0;
    return 0;
}

int ref_upper_f64(const int *arpt, const int *acol, const double *aval, const int *brpt,
                  const int *bcol, const double *bval, int M, int K, int N, int **crpt,
                  int **ccol, double **cval, int *cnnz, int nthreads, double *seconds)
{
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
    Upper_Timing t;
    double t0 = omp_get_wtime();
    brmerge_upper(const_cast<int *>(arpt), const_cast<int *>(acol), const_cast<double *>(aval),
                  const_cast<int *>(brpt), const_cast<int *>(bcol), const_cast<double *>(bval),
                  crpt, ccol, cval, M, K, N, cnnz, t);
    if (seconds)
        *seconds = omp_get_wtime() - t0;
    return 0;
}

// The reference allocates C with new[] (spgemm.h:479, :574-575).
void ref_free_int(int *p) { delete[] p; }
void ref_free_double(double *p) { delete[] p; }
}
