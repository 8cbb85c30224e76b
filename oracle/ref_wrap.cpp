// C entry points around the reference's own brmerge_precise / brmerge_upper
// (BRMerge-SpGEMM/inc/spgemm.h:468-471, :220-223) and its MatrixMarket reader
// (src/CSR.cpp:259-479), compiled from the reference
// sources in place by oracle/build_ref.sh.  Test infrastructure: used to pin
// the oracle restatement and to time the reference on the host cores.
#include "spgemm.h"
#include "CSR.h"

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

// The reference's MatrixMarket reader, CSR::construct (src/CSR.cpp:259-479):
// returns 0 and hands over the CSR arrays (free with ref_free_*), or -1 when
// the reader throws (the message, truncated, goes to msg).  Inputs that reach
// one of the reader's asserts or its unchecked row indexing must not be
// passed here.
int ref_read_mtx(const char *path, int *M, int *N, int *nnz, int **rpt, int **col, double **val,
                 char *msg, int msg_len)
{
    CSR A;
    try {
        A.construct(path);
    } catch (const std::exception &e) {
        if (msg && msg_len > 0) {
            std::strncpy(msg, e.what(), (size_t)msg_len - 1);
            msg[msg_len - 1] = 0;
        }
        return -1;
    }
    *M = A.M;
    *N = A.N;
    *nnz = A.nnz;
    *rpt = A.rpt;
    *col = A.col;
    *val = A.val;
    A.rpt = nullptr;  // ownership moves to the caller
    A.col = nullptr;
    A.val = nullptr;
    return 0;
}
}
