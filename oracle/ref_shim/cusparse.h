/* Host-only stand-in for <cusparse.h>; see cuda_runtime.h in this folder. */
#ifndef SBLAS_REF_SHIM_CUSPARSE_H
#define SBLAS_REF_SHIM_CUSPARSE_H
#include "cuda_runtime.h"
typedef struct sblas_shim_handle *cusparseHandle_t;
typedef struct sblas_shim_descr *cusparseMatDescr_t;
typedef enum {
  CUSPARSE_STATUS_SUCCESS = 0, CUSPARSE_STATUS_NOT_INITIALIZED, CUSPARSE_STATUS_ALLOC_FAILED,
  CUSPARSE_STATUS_INVALID_VALUE, CUSPARSE_STATUS_ARCH_MISMATCH, CUSPARSE_STATUS_MAPPING_ERROR,
  CUSPARSE_STATUS_EXECUTION_FAILED, CUSPARSE_STATUS_INTERNAL_ERROR,
  CUSPARSE_STATUS_MATRIX_TYPE_NOT_SUPPORTED
} cusparseStatus_t;
typedef enum { CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_TRANSPOSE } cusparseOperation_t;
enum { CUSPARSE_MATRIX_TYPE_GENERAL, CUSPARSE_INDEX_BASE_ZERO, CUSPARSE_DIRECTION_ROW,
       CUSPARSE_DIRECTION_COLUMN };
#define SBLAS_SHIM_SPSTUB(name) template <typename... A> static inline cusparseStatus_t name(A &&...) { return CUSPARSE_STATUS_NOT_INITIALIZED; }
SBLAS_SHIM_SPSTUB(cusparseCreate) SBLAS_SHIM_SPSTUB(cusparseDestroy) SBLAS_SHIM_SPSTUB(cusparseSetStream)
SBLAS_SHIM_SPSTUB(cusparseCreateMatDescr) SBLAS_SHIM_SPSTUB(cusparseDestroyMatDescr)
SBLAS_SHIM_SPSTUB(cusparseSetMatType) SBLAS_SHIM_SPSTUB(cusparseSetMatIndexBase)
SBLAS_SHIM_SPSTUB(cusparseDcsrmv) SBLAS_SHIM_SPSTUB(cusparseDcsrmv_mp)
SBLAS_SHIM_SPSTUB(cusparseXcoosort_bufferSizeExt) SBLAS_SHIM_SPSTUB(cusparseCreateIdentityPermutation)
SBLAS_SHIM_SPSTUB(cusparseXcoosortByRow) SBLAS_SHIM_SPSTUB(cusparseXcoosortByColumn)
SBLAS_SHIM_SPSTUB(cusparseDgthr) SBLAS_SHIM_SPSTUB(cusparseXcoo2csr) SBLAS_SHIM_SPSTUB(cusparseDcsc2dense)
SBLAS_SHIM_SPSTUB(cusparseDnnz) SBLAS_SHIM_SPSTUB(cusparseDdense2csr) SBLAS_SHIM_SPSTUB(cusparseDcsr2csc)
#endif
