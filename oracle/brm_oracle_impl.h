/*
 * brm_oracle_impl.h -- value-typed half of the CPU oracle; included twice by
 * brm_oracle.c with BRMO_T = double / float.  Test infrastructure only.
 */
#define BRMO_CAT2(a, b) a##_##b
#define BRMO_CAT(a, b) BRMO_CAT2(a, b)
#define BRMO_FN(name) BRMO_CAT(name, BRMO_SUFFIX)

/* Per-thread ping-pong buffers for the binary row merge. */
typedef struct {
    int *col[2];
    BRMO_T *val[2];
    int *off[2];
} BRMO_FN(brmo_pp);

static void BRMO_FN(brmo_pp_alloc)(BRMO_FN(brmo_pp) * pp, int maxf, int maxk)
{
    size_t nf = (size_t)(maxf > 0 ? maxf : 1), nk = (size_t)maxk + 1;
    for (int s = 0; s < 2; s++) {
        pp->col[s] = (int *)malloc(sizeof(int) * nf);
        pp->val[s] = (BRMO_T *)malloc(sizeof(BRMO_T) * nf);
        pp->off[s] = (int *)malloc(sizeof(int) * nk);
    }
}

static void BRMO_FN(brmo_pp_free)(BRMO_FN(brmo_pp) * pp)
{
    for (int s = 0; s < 2; s++) {
        free(pp->col[s]);
        free(pp->val[s]);
        free(pp->off[s]);
    }
}

/* Merge one C row (spgemm.h:610-709).  Returns the merged length; the
 * result is in pp->col[r]/pp->val[r] where r is written to *res_side. */
static int BRMO_FN(brmo_merge_row)(int i, const int *arpt, const int *acol, const BRMO_T *aval,
                                  const int *brpt, const int *bcol, const BRMO_T *bval,
                                  BRMO_FN(brmo_pp) * pp, int *res_side)
{
    int *dcol = pp->col[0];
    BRMO_T *dval = pp->val[0];
    int *doff = pp->off[0];
    int nlist = 0, n = 0;
    doff[0] = 0;
    /* expand: list l holds row acol[arpt[i]+l] of B scaled by aval */
    for (int j = arpt[i]; j < arpt[i + 1]; j++) {
        BRMO_T a = aval[j];
        int b = acol[j];
        for (int q = brpt[b]; q < brpt[b + 1]; q++) {
            BRMO_T prod = a * bval[q]; /* rounded product (built with -ffp-contract=off) */
            dcol[n] = bcol[q];
            dval[n++] = prod;
        }
        doff[++nlist] = n;
    }
    *res_side = 0;
    if (nlist == 0)
        return 0;
    int src = 0;
    while (nlist != 1) {
        int dst = src ^ 1;
        const int *scol = pp->col[src], *soff = pp->off[src];
        const BRMO_T *sval = pp->val[src];
        int *ocol = pp->col[dst], *ooff = pp->off[dst];
        BRMO_T *oval = pp->val[dst];
        int out_lists = 0, w = 0;
        ooff[0] = 0;
        for (int l = 0; l < nlist; l += 2) {
            if (l + 1 < nlist) {
                int p = soff[l], pe = soff[l + 1];
                int q = soff[l + 1], qe = soff[l + 2];
                while (p < pe && q < qe) {
                    if (scol[p] == scol[q]) {
                        BRMO_T s = sval[p] + sval[q]; /* left + right */
                        ocol[w] = scol[p];
                        oval[w++] = s;
                        p++;
                        q++;
                    } else if (scol[p] < scol[q]) {
                        ocol[w] = scol[p];
                        oval[w++] = sval[p++];
                    } else {
                        ocol[w] = scol[q];
                        oval[w++] = sval[q++];
                    }
                }
                while (p < pe) {
                    ocol[w] = scol[p];
                    oval[w++] = sval[p++];
                }
                while (q < qe) {
                    ocol[w] = scol[q];
                    oval[w++] = sval[q++];
                }
            } else { /* odd last list passes through unchanged */
                for (int p = soff[l]; p < soff[l + 1]; p++) {
                    ocol[w] = scol[p];
                    oval[w++] = sval[p];
                }
            }
            ooff[++out_lists] = w;
        }
        nlist = out_lists;
        src = dst;
    }
    *res_side = src;
    return pp->off[src][1];
}

/* BRMerge-Precise restated (spgemm.h:468-735).  Outputs are malloc'ed. */
int BRMO_FN(brmo_precise)(const int *arpt, const int *acol, const BRMO_T *aval, const int *brpt,
                          const int *bcol, const BRMO_T *bval, int M, int K, int N, int **crpt_,
                          int **ccol_, BRMO_T **cval_, int *cnnz_, int nthreads)
{
    (void)K;
    (void)N;
    int nt = brmo_threads(nthreads);
    size_t m1 = (size_t)(M > 0 ? M : 1);
    int *nnzrA = (int *)malloc(sizeof(int) * m1);
    int *floprC = (int *)malloc(sizeof(int) * m1);
    int *rownnz = (int *)malloc(sizeof(int) * m1);
    long long *scan_flop = (long long *)malloc(sizeof(long long) * ((size_t)M + 1));
    int *sect = (int *)malloc(sizeof(int) * ((size_t)nt + 1));
    int *crpt = (int *)malloc(sizeof(int) * ((size_t)M + 1));

    long long total = brmo_flop(arpt, acol, brpt, M, nnzrA, floprC);
    brmo_scan_i64(floprC, scan_flop, M);
    brmo_sections(scan_flop, M, total, nt, sect);
    brmo_symbolic(arpt, acol, brpt, bcol, floprC, sect, nt, rownnz);

    long long acc = 0;
    crpt[0] = 0;
    for (int i = 0; i < M; i++) {
        acc += rownnz[i];
        if (acc > 2147483647LL) {
            free(nnzrA); free(floprC); free(rownnz); free(scan_flop); free(sect); free(crpt);
            return 5; /* nnz(C) does not fit int32 */
        }
        crpt[i + 1] = (int)acc;
    }
    int cnnz = crpt[M];
    int *ccol = (int *)malloc(sizeof(int) * (size_t)(cnnz > 0 ? cnnz : 1));
    BRMO_T *cval = (BRMO_T *)malloc(sizeof(BRMO_T) * (size_t)(cnnz > 0 ? cnnz : 1));

#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
#else
        int t = 0;
#endif
        int r0 = sect[t], r1 = sect[t + 1];
        int maxf = 0, maxk = 0;
        for (int i = r0; i < r1; i++) {
            if (floprC[i] > maxf) maxf = floprC[i];
            if (nnzrA[i] > maxk) maxk = nnzrA[i];
        }
        BRMO_FN(brmo_pp) pp;
        BRMO_FN(brmo_pp_alloc)(&pp, maxf, maxk);
        for (int i = r0; i < r1; i++) {
            int side;
            int len = BRMO_FN(brmo_merge_row)(i, arpt, acol, aval, brpt, bcol, bval, &pp, &side);
            memcpy(ccol + crpt[i], pp.col[side], sizeof(int) * (size_t)len);
            memcpy(cval + crpt[i], pp.val[side], sizeof(BRMO_T) * (size_t)len);
        }
        BRMO_FN(brmo_pp_free)(&pp);
    }
    free(nnzrA); free(floprC); free(rownnz); free(scan_flop); free(sect);
    *crpt_ = crpt;
    *ccol_ = ccol;
    *cval_ = cval;
    *cnnz_ = cnnz;
    return 0;
}

/* BRMerge-Upper restated (spgemm.h:220-457): merge into an upper-bound
 * buffer at scan_flop offsets, scan the real sizes, then compact. */
int BRMO_FN(brmo_upper)(const int *arpt, const int *acol, const BRMO_T *aval, const int *brpt,
                        const int *bcol, const BRMO_T *bval, int M, int K, int N, int **crpt_,
                        int **ccol_, BRMO_T **cval_, int *cnnz_, int nthreads)
{
    (void)K;
    (void)N;
    int nt = brmo_threads(nthreads);
    size_t m1 = (size_t)(M > 0 ? M : 1);
    int *nnzrA = (int *)malloc(sizeof(int) * m1);
    int *floprC = (int *)malloc(sizeof(int) * m1);
    long long *scan_flop = (long long *)malloc(sizeof(long long) * ((size_t)M + 1));
    int *sect = (int *)malloc(sizeof(int) * ((size_t)nt + 1));
    int *crpt = (int *)malloc(sizeof(int) * ((size_t)M + 1));

    long long total = brmo_flop(arpt, acol, brpt, M, nnzrA, floprC);
    brmo_scan_i64(floprC, scan_flop, M);
    brmo_sections(scan_flop, M, total, nt, sect);

    size_t tot1 = (size_t)(total > 0 ? total : 1);
    int *bar_col = (int *)malloc(sizeof(int) * tot1);
    BRMO_T *bar_val = (BRMO_T *)malloc(sizeof(BRMO_T) * tot1);

#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
#else
        int t = 0;
#endif
        int r0 = sect[t], r1 = sect[t + 1];
        int maxf = 0, maxk = 0;
        for (int i = r0; i < r1; i++) {
            if (floprC[i] > maxf) maxf = floprC[i];
            if (nnzrA[i] > maxk) maxk = nnzrA[i];
        }
        BRMO_FN(brmo_pp) pp;
        BRMO_FN(brmo_pp_alloc)(&pp, maxf, maxk);
        for (int i = r0; i < r1; i++) {
            int side;
            int len = BRMO_FN(brmo_merge_row)(i, arpt, acol, aval, brpt, bcol, bval, &pp, &side);
            memcpy(bar_col + scan_flop[i], pp.col[side], sizeof(int) * (size_t)len);
            memcpy(bar_val + scan_flop[i], pp.val[side], sizeof(BRMO_T) * (size_t)len);
            floprC[i] = len;
        }
        BRMO_FN(brmo_pp_free)(&pp);
    }
    long long acc = 0;
    crpt[0] = 0;
    for (int i = 0; i < M; i++) {
        acc += floprC[i];
        if (acc > 2147483647LL) {
            free(nnzrA); free(floprC); free(scan_flop); free(sect); free(crpt);
            free(bar_col); free(bar_val);
            return 5;
        }
        crpt[i + 1] = (int)acc;
    }
    int cnnz = crpt[M];
    int *ccol = (int *)malloc(sizeof(int) * (size_t)(cnnz > 0 ? cnnz : 1));
    BRMO_T *cval = (BRMO_T *)malloc(sizeof(BRMO_T) * (size_t)(cnnz > 0 ? cnnz : 1));
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int i = 0; i < M; i++) {
        memcpy(ccol + crpt[i], bar_col + scan_flop[i], sizeof(int) * (size_t)floprC[i]);
        memcpy(cval + crpt[i], bar_val + scan_flop[i], sizeof(BRMO_T) * (size_t)floprC[i]);
    }
    free(nnzrA); free(floprC); free(scan_flop); free(sect);
    free(bar_col); free(bar_val);
    *crpt_ = crpt;
    *ccol_ = ccol;
    *cval_ = cval;
    *cnnz_ = cnnz;
    return 0;
}

#undef BRMO_FN
#undef BRMO_CAT
#undef BRMO_CAT2
