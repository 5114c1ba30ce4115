/*
 * oracle.c -- CPU restatement of the reference's FP64 SpMV path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product:
 * only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg
 * and its --impl reference arm) may load liboracle.so.  The library in
 * hpda_sblas_pnnl_gb300/ never links, loads or calls anything here.
 *
 * Every function restates one piece of the reference (JieyangChen7/
 * HPDA_SBLAS_PNNL) and cites the file:line it follows.  The summation order
 * of each loop is the reference's, so the restatement is bit-identical to
 * the reference's own CPU code on the same inputs (checked against the
 * reference's own functions compiled from its sources: oracle/ref_build.sh).
 */
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle.h"

/* test/dspmv_test_smt.cu:39-52 (csr_spmv_cpu): one row at a time,
 * sum += val[j] * x[col[j]] in storage order, then y = alpha*sum + beta*y. */
void oracle_csr_spmv(int m, int n, int nnz, const double *alpha,
                     const double *val, const int *rowptr, const int *col,
                     const double *x, const double *beta, double *y)
{
    (void)n; (void)nnz;
    for (int i = 0; i < m; i++) {
        double sum = 0.0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; j++)
            sum += val[j] * x[col[j]];
        y[i] = (*alpha) * sum + (*beta) * y[i];
    }
}

/* Same loop, rows split statically over OpenMP threads.  Each row keeps the
 * serial order, so the result is bit-identical to oracle_csr_spmv.  This is
 * the timed host baseline (the reference itself has no threaded SpMV; its
 * OpenMP threads only drive GPUs, src/dspmv_mgpu_v1_numa.cu:120). */
void oracle_csr_spmv_omp(int m, int n, int nnz, const double *alpha,
                         const double *val, const int *rowptr, const int *col,
                         const double *x, const double *beta, double *y,
                         int nthreads)
{
    (void)n; (void)nnz;
    const double a = *alpha, b = *beta;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    #pragma omp parallel for schedule(static) num_threads(nthreads)
#else
    (void)nthreads;
#endif
    for (int i = 0; i < m; i++) {
        double sum = 0.0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; j++)
            sum += val[j] * x[col[j]];
        y[i] = a * sum + b * y[i];
    }
}

/* test/dspmv_test_dgx1.cu:55-69 (coo_spmv_cpu): scatter every entry into a
 * zeroed row-sum buffer in storage order, then y = alpha*sum + beta*y. */
void oracle_coo_spmv(int m, int n, int nnz, const double *alpha,
                     const double *val, const int *rowidx, const int *colidx,
                     const double *x, const double *beta, double *y)
{
    (void)n;
    double *sum = (double *)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
    for (int i = 0; i < nnz; i++)
        sum[rowidx[i]] += val[i] * x[colidx[i]];
    for (int i = 0; i < m; i++)
        y[i] = (*alpha) * sum[i] + (*beta) * y[i];
    free(sum);
}

/* CSC form of the same product.  The reference computes it with cuSPARSE
 * csrmv(TRANSPOSE) on the CSC arrays (src/dspmv_mgpu_baseline_csc.cu:131-135),
 * i.e. y = alpha * (A^T)^T x + beta*y; the loop below is the column-order
 * scatter (per column j, sum[row[k]] += val[k]*x[j]). */
void oracle_csc_spmv(int m, int n, int nnz, const double *alpha,
                     const double *val, const int *colptr, const int *rowidx,
                     const double *x, const double *beta, double *y)
{
    (void)nnz;
    double *sum = (double *)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
    for (int j = 0; j < n; j++)
        for (int k = colptr[j]; k < colptr[j + 1]; k++)
            sum[rowidx[k]] += val[k] * x[j];
    for (int i = 0; i < m; i++)
        y[i] = (*alpha) * sum[i] + (*beta) * y[i];
    free(sum);
}

/* ---- compensated "truth" for error reporting -------------------------
 * Dot2 of Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM
 * J. Sci. Comput. 26(6), 2005): TwoProduct by FMA plus TwoSum, giving a
 * row sum as accurate as if computed in twice the working precision.
 * Not a restatement of the reference; used to state each form's error. */
static inline void two_sum(double a, double b, double *s, double *e)
{
    double x = a + b;
    double z = x - a;
    *e = (a - (x - z)) + (b - z);
    *s = x;
}

void oracle_csr_spmv_dot2(int m, int n, int nnz, const double *alpha,
                          const double *val, const int *rowptr, const int *col,
                          const double *x, const double *beta, double *y)
{
    (void)n; (void)nnz;
    for (int i = 0; i < m; i++) {
        double s = 0.0, c = 0.0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; j++) {
            double p = val[j] * x[col[j]];
            double pe = fma(val[j], x[col[j]], -p);
            double t, e;
            two_sum(s, p, &t, &e);
            s = t;
            c += e + pe;
        }
        double row = s + c;
        /* alpha*row + beta*y, also compensated */
        double p1 = (*alpha) * row, e1 = fma(*alpha, row, -p1);
        double p2 = (*beta) * y[i], e2 = fma(*beta, y[i], -p2);
        double t, e;
        two_sum(p1, p2, &t, &e);
        y[i] = t + (e + e1 + e2);
    }
}

/* ---- partition helpers ----------------------------------------------- */

/* src/spmv_helper.cu:18-44 (get_row_from_index): binary search over
 * a[0..n]; returns the last l with a[l] <= idx, except that an exact hit on
 * a[r] at the end returns r.  For a CSR row pointer this is the row that
 * holds nonzero idx, skipping empty rows. */
int oracle_get_row_from_index(int n, const int *a, int idx)
{
    int l = 0, r = n;
    while (l < r - 1) {
        int mid = l + (r - l) / 2;
        if (idx < a[mid]) r = mid;
        else l = mid;
    }
    if (idx == a[l]) return l;
    if (idx == a[r]) return r;
    return l;
}

/* src/spmv_helper.cu:646-665 (findFirstInSorted) */
int oracle_find_first_in_sorted(const int *a, int n, int key)
{
    int l = 0, r = n;
    while (l < r - 1) {
        int mid = l + (r - l) / 2;
        if (key <= a[mid]) r = mid;
        else l = mid;
    }
    if (key == a[l]) return l;
    if (key == a[r]) return r;
    return l;
}

/* src/spmv_helper.cu:668-685 (findLastInSorted) */
int oracle_find_last_in_sorted(const int *a, int n, int key)
{
    int l = 0, r = n;
    while (l < r - 1) {
        int mid = l + (r - l) / 2;
        if (key < a[mid]) r = mid;
        else l = mid;
    }
    if (key == a[l]) return l;
    if (key == a[r]) return r;
    return l;
}

/* ---- multi-part nnz-balanced CSR (the v1 partition + merge) ----------
 * src/dspmv_mgpu_v1.cu:120-193 (split, row lookup, partial-row flags,
 * rebased row pointer) and :304-319 (merge with the partial-row fix).  Each
 * part is computed with the csr loop above on its own rebased arrays, then
 * merged into y exactly as the reference merges device results.  With
 * nparts == 1 this is the reference's single-GPU call.  Used by tests to
 * show that an nnz-balanced split plus a carry merge reproduces the
 * unsplit product (the decomposition the GPU kernels apply inside one GPU).
 * Returns 0, or -1 when a part would be empty (nnz < nparts), a case the
 * reference does not handle. */
/* The v1 partition alone (src/dspmv_mgpu_v1.cu:120-152): for part i,
 * out[7i .. 7i+6] = start_idx, end_idx, start_row, end_row, start_flag,
 * end_flag, dev_m.  Returns -1 when nparts <= 0 or nnz < nparts. */
int oracle_nnz_partition(int m, int nnz, const int *rowptr, int nparts, int *out)
{
    if (nparts <= 0 || nnz < nparts) return -1;
    for (int i = 0; i < nparts; i++) {
        int *o = out + 7 * i;
        o[0] = (int)floor((double)((long long)i * nnz) / nparts);
        o[1] = (int)floor((double)((long long)(i + 1) * nnz) / nparts) - 1;
        o[2] = oracle_get_row_from_index(m, rowptr, o[0]);
        o[3] = oracle_get_row_from_index(m, rowptr, o[1]);
        o[4] = o[0] > rowptr[o[2]];
        o[5] = o[1] < rowptr[o[3] + 1] - 1;
        o[6] = o[3] - o[2] + 1;
    }
    return 0;
}

int oracle_csr_spmv_nnz_split(int m, int n, int nnz, const double *alpha,
                              const double *val, const int *rowptr, const int *col,
                              const double *x, const double *beta, double *y,
                              int nparts)
{
    if (nparts <= 0 || nnz < nparts) return -1;
    int *start_idx = (int *)malloc(sizeof(int) * nparts);
    int *end_idx = (int *)malloc(sizeof(int) * nparts);
    int *start_row = (int *)malloc(sizeof(int) * nparts);
    int *end_row = (int *)malloc(sizeof(int) * nparts);
    int *start_flag = (int *)malloc(sizeof(int) * nparts);
    double *y2 = (double *)malloc(sizeof(double) * nparts);
    for (int i = 0; i < nparts; i++) {
        /* :122-129 -- floor(i*nnz/ngpu) in double (64-bit product here) */
        start_idx[i] = (int)floor((double)((long long)i * nnz) / nparts);
        end_idx[i] = (int)floor((double)((long long)(i + 1) * nnz) / nparts) - 1;
    }
    for (int i = 0; i < nparts; i++) {            /* :132-142 */
        start_row[i] = oracle_get_row_from_index(m, rowptr, start_idx[i]);
        start_flag[i] = start_idx[i] > rowptr[start_row[i]];
        if (start_flag[i]) y2[i] = y[start_row[i]];
    }
    for (int i = 0; i < nparts; i++)              /* :143-152 */
        end_row[i] = oracle_get_row_from_index(m, rowptr, end_idx[i]);

    /* every part copies its rows of the caller's y before any merge (:242) */
    double *y0 = (double *)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
    memcpy(y0, y, sizeof(double) * (size_t)m);
    for (int d = 0; d < nparts; d++) {
        int dm = end_row[d] - start_row[d] + 1;
        int dnnz = end_idx[d] - start_idx[d] + 1;
        int *prow = (int *)malloc(sizeof(int) * (dm + 1));
        /* :186-192 -- first entry 0, last entry dev_nnz, inner rows rebased */
        prow[0] = 0;
        prow[dm] = dnnz;
        for (int j = 1; j < dm; j++) prow[j] = rowptr[start_row[d] + j] - start_idx[d];
        double *py = (double *)malloc(sizeof(double) * dm);
        memcpy(py, y0 + start_row[d], sizeof(double) * dm);
        oracle_csr_spmv(dm, n, dnnz, alpha, val + start_idx[d], prow, col + start_idx[d],
                        x, beta, py);
        /* :304-319 -- copy the part back, then for a row split with the
         * previous part add back the previous part's value and remove the
         * second beta*y0 term */
        double tmp = 0.0;
        if (start_flag[d]) tmp = y[start_row[d]];
        memcpy(y + start_row[d], py, sizeof(double) * dm);
        if (start_flag[d]) {
            y[start_row[d]] += tmp;
            y[start_row[d]] -= y2[d] * (*beta);
        }
        free(prow);
        free(py);
    }
    free(start_idx); free(end_idx); free(start_row); free(end_row);
    free(start_flag); free(y2); free(y0);
    return 0;
}

/* ---- the reference's 'g' matrix ------------------------------------------
 * test/dspmv_test_smt.cu:176-232: n x n, nb = n/8 row blocks; rows of the
 * first block hold columns 0..ceil(0.9n)-1, all other rows columns
 * 0..ceil(0.01n)-1; all values 1.0, written as row-major COO.  Returns nnz
 * and fills the arrays when they are non-NULL.  Like the reference, the
 * generator walks whole blocks, so n must be a multiple of 8 (otherwise the
 * reference writes rows past n); -1 is returned in that case. */
long long oracle_gen_g(int n, int *rowidx, int *colidx, double *val)
{
    if (n <= 0 || n % 8 != 0) return -1;
    int m = n, nb = m / 8;
    long long p = 0;
    for (int i = 0; i < m; i += nb) {
        double r = (i == 0) ? 0.9 : 0.01;
        for (int ii = i; ii < i + nb; ii++) {
            for (int j = 0; j < n * r; j++) {     /* j < n*r in double, as :215 */
                if (rowidx) { rowidx[p] = ii; colidx[p] = j; val[p] = 1.0; }
                p++;
            }
        }
    }
    return p;
}

/* ---- COO -> CSR / CSC on the host --------------------------------------
 * Result format of the reference's coo2csr / coo2csc
 * (src/spmv_helper.cu:493-572, :575-642): a stable sort by row (by column for
 * CSC) of the COO triplets, then the compressed pointer.  cuSPARSE coosort
 * is a stable radix sort of the keys, so entries with the same row keep
 * their input order.  Restated with a counting sort. */
static void counting_sort_compress(int nkeys, int nnz, const int *key, const int *other,
                                   const double *val, int *ptr, int *other_out,
                                   double *val_out)
{
    memset(ptr, 0, sizeof(int) * (size_t)(nkeys + 1));
    for (int k = 0; k < nnz; k++) ptr[key[k] + 1]++;
    for (int i = 0; i < nkeys; i++) ptr[i + 1] += ptr[i];
    int *cur = (int *)malloc(sizeof(int) * (size_t)(nkeys > 0 ? nkeys : 1));
    memcpy(cur, ptr, sizeof(int) * (size_t)nkeys);
    for (int k = 0; k < nnz; k++) {
        int d = cur[key[k]]++;
        other_out[d] = other[k];
        val_out[d] = val[k];
    }
    free(cur);
}

void oracle_coo2csr(int m, int n, int nnz, const double *cooval, const int *coorow,
                    const int *coocol, double *csrval, int *csrrowptr, int *csrcol)
{
    (void)n;
    counting_sort_compress(m, nnz, coorow, coocol, cooval, csrrowptr, csrcol, csrval);
}

void oracle_coo2csc(int m, int n, int nnz, const double *cooval, const int *coorow,
                    const int *coocol, double *cscval, int *csccolptr, int *cscrow)
{
    (void)m;
    counting_sort_compress(n, nnz, coocol, coorow, cooval, csccolptr, cscrow, cscval);
}

/* Several right-hand sides: the csr_spmv_cpu loop (test/dspmv_test_smt.cu:39-52)
 * applied to every column c of a row-major X (n x k, row stride ldx) into Y
 * (m x k, row stride ldy), same per-row summation order.  The reference has
 * no SpMM; its task pool (src/dspmv_mgpu_v2.cu:103-307) runs independent
 * products, which this restates column by column.  val == NULL: every stored
 * entry is 1 (pattern-only matrices). */
void oracle_csr_spmm(int m, int n, int k, const double *alpha, const double *val,
                     const int *rowptr, const int *col, const double *x, int ldx,
                     const double *beta, double *y, int ldy, int nthreads)
{
    (void)n;
    const double a = *alpha, b = *beta;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    #pragma omp parallel for schedule(static) num_threads(nthreads)
#else
    (void)nthreads;
#endif
    for (int i = 0; i < m; i++) {
        for (int c = 0; c < k; c++) {
            double sum = 0.0;
            for (int j = rowptr[i]; j < rowptr[i + 1]; j++)
                sum += (val ? val[j] : 1.0) * x[(long long)col[j] * ldx + c];
            y[(long long)i * ldy + c] = a * sum + b * y[(long long)i * ldy + c];
        }
    }
}

/* Adjoint of Y = A X with respect to X (no counterpart in the reference):
 * dX = A^T G, scattered row by row in storage order (dX overwritten). */
void oracle_csr_spmm_t(int m, int n, int k, const double *val, const int *rowptr,
                       const int *col, const double *g, int ldg, double *dx, int lddx)
{
    for (int j = 0; j < n; j++)
        for (int c = 0; c < k; c++) dx[(long long)j * lddx + c] = 0.0;
    for (int i = 0; i < m; i++)
        for (int p = rowptr[i]; p < rowptr[i + 1]; p++)
            for (int c = 0; c < k; c++)
                dx[(long long)col[p] * lddx + c] += (val ? val[p] : 1.0) * g[(long long)i * ldg + c];
}

/* Adjoint of Y = A X with respect to the stored values (no counterpart in
 * the reference): dval[p] = sum over c of G[row(p), c] * X[col(p), c]. */
void oracle_csr_sddmm(int m, int k, const int *rowptr, const int *col, const double *g, int ldg,
                      const double *x, int ldx, double *dval)
{
    for (int i = 0; i < m; i++)
        for (int p = rowptr[i]; p < rowptr[i + 1]; p++) {
            double s = 0.0;
            for (int c = 0; c < k; c++)
                s += g[(long long)i * ldg + c] * x[(long long)col[p] * ldx + c];
            dval[p] = s;
        }
}

/* The x-zero filter of spMspV_mgpu_v1 / _v2 (src/dspmv_mgpu_v1.cu:29-40,
 * src/dspmv_mgpu_v2.cu:55-65): keep the nonzeros j of every row with
 * x[col[j]] != 0.0, in storage order; returns the kept count. */
long long oracle_csr_filter_x(int m, const int *rowptr, const int *col, const double *val,
                              const double *x, int *orowptr, int *ocol, double *oval)
{
    long long k = 0;
    orowptr[0] = 0;
    for (int i = 0; i < m; i++) {
        for (int j = rowptr[i]; j < rowptr[i + 1]; j++)
            if (x[col[j]] != 0.0) {
                oval[k] = val[j];
                ocol[k] = col[j];
                k++;
            }
        orowptr[i + 1] = (int)k;
    }
    return k;
}

/* The reference's reading of a coordinate MatrixMarket file
 * (test/dspmv_test_dgx1.cu:133-181): the banner's type word, the size line
 * after the '%' comment lines ("M N nz", as the NIST mm_read_mtx_crd_size
 * reads it), then one fscanf per entry: "%d %d\n" for pattern files (value
 * 1), "%d %d %lg\n" for real, "%d %d %d\n" for integer (converted to
 * double), both indices minus one.  With row, col and val NULL only the
 * header is read (*kind: 0 real, 1 integer, 2 pattern).  Returns 0, or -1
 * when the file, its header or an entry cannot be read (the reference
 * ignores fscanf's result; on well-formed files the two agree). */
int oracle_mm_read_fscanf(const char *path, int *m, int *n, long long *nnz, int *kind,
                          int *row, int *col, double *val)
{
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    char line[1025];
    if (!fgets(line, sizeof line, f) || strncmp(line, "%%MatrixMarket", 14) != 0) {
        fclose(f);
        return -1;
    }
    for (char *p = line; *p; ++p) *p = (char)tolower((unsigned char)*p);
    *kind = strstr(line, "pattern") ? 2 : (strstr(line, "integer") ? 1 : 0);
    do {
        if (!fgets(line, sizeof line, f)) {
            fclose(f);
            return -1;
        }
    } while (line[0] == '%');
    int mm = 0, nn = 0, nz = 0;
    if (sscanf(line, "%d %d %d", &mm, &nn, &nz) != 3) {
        fclose(f);
        return -1;
    }
    *m = mm;
    *n = nn;
    *nnz = nz;
    if (!row || !col || !val) {
        fclose(f);
        return 0;
    }
    for (int i = 0; i < nz; i++) {
        int ok;
        if (*kind == 2) {
            ok = fscanf(f, "%d %d\n", &row[i], &col[i]) == 2;
            val[i] = 1;
        } else if (*kind == 0) {
            ok = fscanf(f, "%d %d %lg\n", &row[i], &col[i], &val[i]) == 3;
        } else {
            int tmp = 0;
            ok = fscanf(f, "%d %d %d\n", &row[i], &col[i], &tmp) == 3;
            val[i] = tmp;
        }
        if (!ok) {
            fclose(f);
            return -1;
        }
        row[i]--;
        col[i]--;
    }
    fclose(f);
    return 0;
}
