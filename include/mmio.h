/*
 * mmio.h -- MatrixMarket entry points of libsblas_gb300.so.
 *
 * The reference's drivers read their matrices with the NIST MatrixMarket
 * I/O routines declared in its include/mmio.h (mm_read_banner,
 * mm_read_mtx_crd_size, mm_typecode_to_str and the mm_is_* queries; used at
 * test/dspmv_test_dgx1.cu:133-181, dspmv_test_dgx2.cu, dspmv_test_smt.cu).
 * The reference vendors them header-only: its include/mmio.h holds the
 * declarations and the function bodies (mm_read_banner at :254,
 * mm_read_mtx_crd_size at :339), compiled into every driver that includes
 * it.  This header keeps that interface (the MM_typecode layout, query macros, error codes
 * and signatures are the published NIST ones, so a driver compiles
 * unchanged) with C linkage, implemented by the library.
 *
 * It adds a multi-threaded reader of a whole coordinate file into COO
 * arrays (sblas_mm_read_header / sblas_mm_read_coo), the replacement of the
 * drivers' per-entry fscanf loop.
 */
#ifndef SBLAS_MMIO_H
#define SBLAS_MMIO_H

#include <stdio.h>
#include "sblas_gb300.h"

#define MM_MAX_LINE_LENGTH 1025
#define MatrixMarketBanner "%%MatrixMarket"
#define MM_MAX_TOKEN_LENGTH 64

/* [0] 'M' matrix; [1] 'C' coordinate / 'A' array; [2] 'R' real, 'C'
 * complex, 'P' pattern, 'I' integer; [3] 'G' general, 'S' symmetric, 'H'
 * hermitian, 'K' skew-symmetric. */
typedef char MM_typecode[4];

#define mm_is_matrix(typecode) ((typecode)[0] == 'M')
#define mm_is_sparse(typecode) ((typecode)[1] == 'C')
#define mm_is_coordinate(typecode) ((typecode)[1] == 'C')
#define mm_is_dense(typecode) ((typecode)[1] == 'A')
#define mm_is_array(typecode) ((typecode)[1] == 'A')
#define mm_is_complex(typecode) ((typecode)[2] == 'C')
#define mm_is_real(typecode) ((typecode)[2] == 'R')
#define mm_is_pattern(typecode) ((typecode)[2] == 'P')
#define mm_is_integer(typecode) ((typecode)[2] == 'I')
#define mm_is_symmetric(typecode) ((typecode)[3] == 'S')
#define mm_is_general(typecode) ((typecode)[3] == 'G')
#define mm_is_skew(typecode) ((typecode)[3] == 'K')
#define mm_is_hermitian(typecode) ((typecode)[3] == 'H')

/* return codes of the mm_* routines (0 = success) */
#define MM_COULD_NOT_READ_FILE 11
#define MM_PREMATURE_EOF 12
#define MM_NOT_MTX 13
#define MM_NO_HEADER 14
#define MM_UNSUPPORTED_TYPE 15
#define MM_LINE_TOO_LONG 16
#define MM_COULD_NOT_WRITE_FILE 17

#ifdef __cplusplus
extern "C" {
#endif

/* Reads the banner line "%%MatrixMarket matrix <coordinate|array>
 * <real|complex|pattern|integer> <general|symmetric|hermitian|
 * skew-symmetric>" (tokens after the first case-insensitive). */
SBLAS_API int mm_read_banner(FILE *f, MM_typecode *matcode);

/* Skips comment lines ('%') and reads "M N nz". */
SBLAS_API int mm_read_mtx_crd_size(FILE *f, int *M, int *N, int *nz);

/* Skips comment lines ('%') and reads "M N" (dense array files). */
SBLAS_API int mm_read_mtx_array_size(FILE *f, int *M, int *N);

/* 1 when the type combination is one the format allows. */
SBLAS_API int mm_is_valid(MM_typecode matcode);

/* "matrix coordinate real general" and so on, in memory from malloc (the
 * caller may free it); NULL for an invalid code. */
SBLAS_API char *mm_typecode_to_str(MM_typecode matcode);

/* ---- whole-file reader (no counterpart in the reference) --------------- */

typedef struct sblas_mm_header {
    int m;               /* rows */
    int n;               /* columns */
    long long nnz;       /* stored entries announced by the size line */
    char typecode[4];    /* MM_typecode */
    int reserved;
} sblas_mm_header;

/* Banner and size line of a coordinate file.  Complex and dense (array)
 * files fail with SBLAS_ERR_UNSUPPORTED, a malformed header with
 * SBLAS_ERR_FORMAT. */
SBLAS_API int sblas_mm_read_header(const char *path, sblas_mm_header *h);

/* Reads the entries of a coordinate file into COO arrays, 0-based, in file
 * order, using nthreads host threads (0: all cores).  The results equal the
 * reference's test programs' loop (test/dspmv_test_dgx1.cu:160-181): rows and
 * columns minus one; real values as strtod reads them (fscanf "%lg");
 * integer values converted to double; pattern values 1.0; the first nnz
 * entries of the file (later lines ignored; fewer is an error).
 *
 * expand_symmetric = 0 keeps the stored triangle only, as the reference
 * does.  With 1, a symmetric or hermitian (real) file also yields (j, i, v)
 * for every stored off-diagonal (i, j, v), skew-symmetric (j, i, -v); the
 * mirrored entries follow the stored ones, in file order.
 *
 * *count receives the number of entries written (or needed).  With row,
 * col and val all NULL nothing is written (the size query); otherwise cap
 * must be at least that number (SBLAS_ERR_ARG otherwise).  One entry per
 * line; blank lines and lines starting with '%' are skipped; an index out
 * of range, a missing or unreadable token fails with SBLAS_ERR_FORMAT and
 * the line number in sblas_last_error(). */
SBLAS_API int sblas_mm_read_coo(const char *path, int expand_symmetric, int nthreads,
                                long long cap, int *row, int *col, double *val,
                                long long *count);

#ifdef __cplusplus
}
#endif

#endif /* SBLAS_MMIO_H */
