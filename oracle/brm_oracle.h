/*
 * brm_oracle.h -- CPU restatement of BRMerge SpGEMM used as the parity oracle
 * and as the timed CPU baseline.  TEST INFRASTRUCTURE: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs may load it.
 *
 * All outputs are malloc'ed; release them with brmo_free().
 * nthreads <= 0 means all OpenMP threads.  Return 0 on success, 5 when
 * nnz(C) does not fit int32.
 */
#ifndef BRM_ORACLE_H
#define BRM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

int brmo_precise_f64(const int *arpt, const int *acol, const double *aval, const int *brpt,
                     const int *bcol, const double *bval, int M, int K, int N, int **crpt,
                     int **ccol, double **cval, int *cnnz, int nthreads);
int brmo_upper_f64(const int *arpt, const int *acol, const double *aval, const int *brpt,
                   const int *bcol, const double *bval, int M, int K, int N, int **crpt,
                   int **ccol, double **cval, int *cnnz, int nthreads);
int brmo_precise_f32(const int *arpt, const int *acol, const float *aval, const int *brpt,
                     const int *bcol, const float *bval, int M, int K, int N, int **crpt,
                     int **ccol, float **cval, int *cnnz, int nthreads);
int brmo_upper_f32(const int *arpt, const int *acol, const float *aval, const int *brpt,
                   const int *bcol, const float *bval, int M, int K, int N, int **crpt,
                   int **ccol, float **cval, int *cnnz, int nthreads);
long long brmo_compute_flop(const int *arpt, const int *acol, const int *brpt, int M);
void brmo_row_flops(const int *arpt, const int *acol, const int *brpt, int M, int *floprC);
void brmo_free(void *p);
int brmo_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
