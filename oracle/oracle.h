/*
 * oracle.h -- CPU restatement of the reference's FP64 SpMV path.
 * TEST INFRASTRUCTURE ONLY (see oracle.c); never part of the product.
 */
#ifndef SBLAS_ORACLE_H
#define SBLAS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

void oracle_csr_spmv(int m, int n, int nnz, const double *alpha,
                     const double *val, const int *rowptr, const int *col,
                     const double *x, const double *beta, double *y);
void oracle_csr_spmv_omp(int m, int n, int nnz, const double *alpha,
                         const double *val, const int *rowptr, const int *col,
                         const double *x, const double *beta, double *y,
                         int nthreads);
void oracle_coo_spmv(int m, int n, int nnz, const double *alpha,
                     const double *val, const int *rowidx, const int *colidx,
                     const double *x, const double *beta, double *y);
void oracle_csc_spmv(int m, int n, int nnz, const double *alpha,
                     const double *val, const int *colptr, const int *rowidx,
                     const double *x, const double *beta, double *y);
void oracle_csr_spmv_dot2(int m, int n, int nnz, const double *alpha,
                          const double *val, const int *rowptr, const int *col,
                          const double *x, const double *beta, double *y);

int oracle_get_row_from_index(int n, const int *a, int idx);
int oracle_find_first_in_sorted(const int *a, int n, int key);
int oracle_find_last_in_sorted(const int *a, int n, int key);

int oracle_nnz_partition(int m, int nnz, const int *rowptr, int nparts, int *out);
int oracle_csr_spmv_nnz_split(int m, int n, int nnz, const double *alpha,
                              const double *val, const int *rowptr, const int *col,
                              const double *x, const double *beta, double *y,
                              int nparts);

long long oracle_gen_g(int n, int *rowidx, int *colidx, double *val);

void oracle_coo2csr(int m, int n, int nnz, const double *cooval, const int *coorow,
                    const int *coocol, double *csrval, int *csrrowptr, int *csrcol);
void oracle_coo2csc(int m, int n, int nnz, const double *cooval, const int *coorow,
                    const int *coocol, double *cscval, int *csccolptr, int *cscrow);

void oracle_csr_spmm(int m, int n, int k, const double *alpha, const double *val,
                     const int *rowptr, const int *col, const double *x, int ldx,
                     const double *beta, double *y, int ldy, int nthreads);
void oracle_csr_spmm_t(int m, int n, int k, const double *val, const int *rowptr,
                       const int *col, const double *g, int ldg, double *dx, int lddx);
void oracle_csr_sddmm(int m, int k, const int *rowptr, const int *col, const double *g, int ldg,
                      const double *x, int ldx, double *dval);
long long oracle_csr_filter_x(int m, const int *rowptr, const int *col, const double *val,
                              const double *x, int *orowptr, int *ocol, double *oval);

/* test/dspmv_test_dgx1.cu:133-181: per-entry fscanf reading of a coordinate
 * file (header query with NULL arrays). */
int oracle_mm_read_fscanf(const char *path, int *m, int *n, long long *nnz, int *kind,
                          int *row, int *col, double *val);

#ifdef __cplusplus
}
#endif
#endif
