/* Exports the reference's own CPU functions, compiled from its sources by
 * oracle/ref_build.sh, under C names for ctypes.  These declarations repeat
 * the reference's signatures (test/dspmv_test_smt.cu:39-44,
 * test/dspmv_test_dgx1.cu:55-57, include/spmv_kernel.h:300,348-349). */
void csr_spmv_cpu(int m, int n, int nnz, double *alpha, double *cooVal, int *csrRowPtr,
                  int *cooColIndex, double *x, double *beta, double *y);
void coo_spmv_cpu(int m, int n, int nnz, double *alpha, double *cooVal, int *cooRowIdx,
                  int *cooColIdx, double *x, double *beta, double *y);
int get_row_from_index(int n, int *a, int idx);
int findFirstInSorted(int *a, int n, int key);
int findLastInSorted(int *a, int n, int key);

extern "C" {
void ref_csr_spmv_cpu(int m, int n, int nnz, double *alpha, double *val, int *rowptr,
                      int *col, double *x, double *beta, double *y)
{ csr_spmv_cpu(m, n, nnz, alpha, val, rowptr, col, x, beta, y); }
void ref_coo_spmv_cpu(int m, int n, int nnz, double *alpha, double *val, int *row,
                      int *col, double *x, double *beta, double *y)
{ coo_spmv_cpu(m, n, nnz, alpha, val, row, col, x, beta, y); }
int ref_get_row_from_index(int n, int *a, int idx) { return get_row_from_index(n, a, idx); }
int ref_find_first_in_sorted(int *a, int n, int key) { return findFirstInSorted(a, n, key); }
int ref_find_last_in_sorted(int *a, int n, int key) { return findLastInSorted(a, n, key); }
}

#include <omp.h>
extern "C" {
/* The reference's serial csr_spmv_cpu run on contiguous row slices by
 * nthreads OpenMP threads (each slice is a valid call: the row pointer keeps
 * absolute offsets into val/col).  Per-row arithmetic is the reference's. */
void ref_csr_spmv_cpu_threads(int m, int n, int nnz, double *alpha, double *val, int *rowptr,
                              int *col, double *x, double *beta, double *y, int nthreads)
{
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    #pragma omp parallel num_threads(nthreads)
    {
        int t = omp_get_thread_num(), nt = omp_get_num_threads();
        int r0 = (int)((long long)m * t / nt), r1 = (int)((long long)m * (t + 1) / nt);
        if (r1 > r0) csr_spmv_cpu(r1 - r0, n, nnz, alpha, val, rowptr + r0, col, x, beta, y + r0);
    }
}
}
