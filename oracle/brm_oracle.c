/*
 * brm_oracle.c -- CPU restatement of BRMerge SpGEMM (C = A*B, CSR, int32 indices).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline
 * and reference legs) load it, and only as the checker.  The product library
 * (brmerge_gb300/csrc, libbrmerge.so) never links, loads or calls it.
 *
 * Parity pin: this restatement is checked bit-for-bit against the reference's
 * own brmerge_precise / brmerge_upper, compiled unmodified from the reference
 * sources by oracle/build_ref.sh, on committed golden fixtures
 * (tests/golden/, produced by tests/golden/make_golden.py) and on seeded
 * random inputs (tests/test_oracle.py).
 *
 * Algorithm (restated from BRMerge-SpGEMM/inc/spgemm.h; same phases):
 *   1. per-row products   floprC[i] = sum_j nnz(B(acol[j],:))   spgemm.h:31-56
 *   2. exclusive scan of floprC into int64                      spgemm.h:138-187, :490
 *   3. static flop-balanced row ranges per thread               spgemm.h:189-215, :496-503
 *   4. symbolic: linear-probing hash, size upper_log(flop),
 *      hash = (col*107) & (size-1), empty = -1                  spgemm.h:505-562, :69-80
 *   5. crpt = exclusive scan of the row nnz                     spgemm.h:564-578
 *   6. numeric: per row, expand list l = (bcol, aval*bval) for
 *      the l-th A entry (empty B rows still make an empty list),
 *      then merge adjacent pairs (0,1),(2,3).. copying an odd
 *      last list, ping-pong until one list is left; equal columns
 *      are summed src1 + src2 (left list first)                 spgemm.h:580-721
 *   Upper: steps 1-3, numeric into a per-row buffer at scan_flop
 *      offsets, scan of the real row sizes, compaction copy     spgemm.h:220-457
 *
 * The arithmetic is a product a*b rounded to the value type, then sums of
 * two rounded values; build with -ffp-contract=off so that no product is
 * fused into a sum (the reference stores the product before adding it).
 * The value type is a macro parameter: the file is compiled twice through
 * brm_oracle_impl.h (double and float entry points).
 */
#include "brm_oracle.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- shared integer helpers (value-type independent) ---------------------- */

/* Smallest power of two >= num, with upper_log(0) == 2 (spgemm.h:69-80). */
static int brmo_upper_pow2(int num)
{
    int base = 0;
    int a = num;
    while ((a >>= 1) != 0)
        base++;
    if (num != (1 << base))
        return 1 << (base + 1);
    return 1 << base;
}

/* Row products and A-row lengths; returns the int64 total (spgemm.h:31-56). */
static long long brmo_flop(const int *arpt, const int *acol, const int *brpt, int M,
                           int *nnzrA, int *floprC)
{
    long long total = 0;
#pragma omp parallel for reduction(+ : total) schedule(static)
    for (int i = 0; i < M; i++) {
        long long s = 0;
        nnzrA[i] = arpt[i + 1] - arpt[i];
        for (int j = arpt[i]; j < arpt[i + 1]; j++)
            s += brpt[acol[j] + 1] - brpt[acol[j]];
        floprC[i] = (int)s;
        total += s;
    }
    return total;
}

/* Exclusive scan with out[n] = total. */
static void brmo_scan_i64(const int *in, long long *out, int n)
{
    out[0] = 0;
    for (int i = 0; i < n; i++)
        out[i + 1] = out[i] + in[i];
}

/* Index of the last entry <= key in the non-decreasing arr[0..n) (arr[0] <= key). */
static int brmo_last_le(const long long *arr, int n, long long key)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = lo + (hi - lo + 1) / 2;
        if (arr[mid] <= key)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

/* Row ranges with about equal products per thread (spgemm.h:496-503). */
static void brmo_sections(const long long *scan_flop, int M, long long total, int nthreads,
                          int *sect)
{
    sect[0] = 0;
    for (int t = 1; t < nthreads; t++) {
        long long target = (long long)((double)total / nthreads * t);
        sect[t] = brmo_last_le(scan_flop, M + 1, target);
        if (sect[t] > M)
            sect[t] = M;
        if (sect[t] < sect[t - 1])
            sect[t] = sect[t - 1];
    }
    sect[nthreads] = M;
}

static int brmo_threads(int requested)
{
#ifdef _OPENMP
    return requested > 0 ? requested : omp_get_max_threads();
#else
    (void)requested;
    return 1;
#endif
}

/* Exact nnz per C row by linear-probing hash (spgemm.h:505-562).
 * Writes the counts into nnz[]. */
static void brmo_symbolic(const int *arpt, const int *acol, const int *brpt, const int *bcol,
                          const int *floprC, const int *sect, int nthreads, int *nnz)
{
#pragma omp parallel num_threads(nthreads)
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
#else
        int t = 0;
#endif
        int r0 = sect[t], r1 = sect[t + 1];
        int maxf = 0;
        for (int i = r0; i < r1; i++)
            if (floprC[i] > maxf)
                maxf = floprC[i];
        int tsize = brmo_upper_pow2(maxf);
        int *ht = (int *)malloc(sizeof(int) * (size_t)tsize);
        for (int i = r0; i < r1; i++) {
            int size = brmo_upper_pow2(floprC[i]);
            int mask = size - 1;
            for (int s = 0; s < size; s++)
                ht[s] = -1;
            int count = 0;
            for (int j = arpt[i]; j < arpt[i + 1]; j++) {
                int b = acol[j];
                for (int q = brpt[b]; q < brpt[b + 1]; q++) {
                    int key = bcol[q];
                    int h = (int)(((unsigned)key * 107u) & (unsigned)mask);
                    for (;;) {
                        if (ht[h] == key)
                            break;
                        if (ht[h] == -1) {
                            ht[h] = key;
                            count++;
                            break;
                        }
                        h = (h + 1) & mask;
                    }
                }
            }
            nnz[i] = count;
        }
        free(ht);
    }
}

/* ---- value-typed parts --------------------------------------------------- */

#define BRMO_T double
#define BRMO_SUFFIX f64
#include "brm_oracle_impl.h"
#undef BRMO_T
#undef BRMO_SUFFIX

#define BRMO_T float
#define BRMO_SUFFIX f32
#include "brm_oracle_impl.h"
#undef BRMO_T
#undef BRMO_SUFFIX

long long brmo_compute_flop(const int *arpt, const int *acol, const int *brpt, int M)
{
    int *nnzrA = (int *)malloc(sizeof(int) * (size_t)(M > 0 ? M : 1));
    int *floprC = (int *)malloc(sizeof(int) * (size_t)(M > 0 ? M : 1));
    long long f = brmo_flop(arpt, acol, brpt, M, nnzrA, floprC);
    free(nnzrA);
    free(floprC);
    return f;
}

void brmo_row_flops(const int *arpt, const int *acol, const int *brpt, int M, int *floprC)
{
    int *nnzrA = (int *)malloc(sizeof(int) * (size_t)(M > 0 ? M : 1));
    brmo_flop(arpt, acol, brpt, M, nnzrA, floprC);
    free(nnzrA);
}

void brmo_free(void *p) { free(p); }

int brmo_max_threads(void) { return brmo_threads(0); }
