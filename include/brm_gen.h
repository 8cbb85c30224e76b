/*
 * brm_gen.h -- deterministic synthetic CSR generators (host, C ABI).
 *
 * The reference ships no matrices (its drivers read MatrixMarket files,
 * BRMerge-SpGEMM/src/brmerge_precise.cpp:17-39, and its R-MAT header is
 * absent); these generators stand in for its inputs with seeded, documented
 * distributions.  The PRNG is xoshiro256** seeded through splitmix64, so the
 * integer structure is identical on every host.
 *
 * Every generator fills a brm_host_csr whose arrays are malloc'ed; release it
 * with brm_host_csr_free().  Columns are sorted and unique within each row.
 * Return 0 on success, 1 on a bad argument, 3 when memory runs out.
 */
#ifndef BRM_GEN_H
#define BRM_GEN_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct brm_host_csr {
    int M, N, nnz;
    int *rpt;    /* M+1 */
    int *col;    /* nnz */
    double *val; /* nnz */
} brm_host_csr;

void brm_host_csr_free(brm_host_csr *m);

/* Erdos-Renyi: exactly per_row distinct uniform columns per row, values U[-1,1]. */
int brm_gen_er(int n, int per_row, unsigned long long seed, brm_host_csr *out);

/* R-MAT (a,b,c,d=1-a-b-c) on 2^scale x 2^scale with `edges` samples,
 * duplicates removed, values U[-1,1]. */
int brm_gen_rmat(int scale, long long edges, double a, double b, double c,
                 unsigned long long seed, brm_host_csr *out);

/* 27-point stencil on an nx*ny*nz grid: 26 on the diagonal, -1 off it, each
 * entry plus U[-jitter, jitter]. */
int brm_gen_stencil27(int nx, int ny, int nz, double jitter, unsigned long long seed,
                      brm_host_csr *out);

/* M x N with row lengths round(lognormal(mu, sigma)) capped at min(cap, N),
 * uniform random distinct columns, values U[-1,1]. */
int brm_gen_lognormal(int M, int N, double mu, double sigma, int cap,
                      unsigned long long seed, brm_host_csr *out);

/* M x N where each row length is uniform in [0, max_per_row] (capped at N),
 * uniform random distinct columns in [0, N), values U[-1,1]. */
int brm_gen_uniform(int M, int N, int max_per_row, unsigned long long seed, brm_host_csr *out);

/* Host builds of the device MatrixMarket token parsers (brm_read_mtx*), for
 * testing them without a GPU.  Status 0: converted (correctly rounded);
 * 1: valid, but the device defers the value to an exact host conversion;
 * -1: not a number of the reader's grammar. */
int brm_parse_int_token(const char *s, int len, long long *out);
int brm_parse_real_token(const char *s, int len, double *out);
void brm_parse_real_tokens(const char *buf, const long long *off, const int *len, long long n,
                           double *out, int *status);

#ifdef __cplusplus
}
#endif
#endif
