/*
 * spmv_kernel.h -- drop-in boundary of libsblas_gb300.so.
 *
 * Same entry points, argument order and meaning as the reference's
 * include/spmv_kernel.h (JieyangChen7/HPDA_SBLAS_PNNL), exported with C
 * linkage so that C, C++, ctypes, cgo or JNI callers bind them by name.  A
 * C++ driver written against the reference header compiles unchanged
 * against this one (spmv_ret keeps its member functions under C++).
 *
 * Ownership and threading follow the reference: every array argument of the
 * spMV_* entry points is a HOST pointer (pinned or pageable), alpha and beta
 * point to host doubles, y is read (when beta != 0) and overwritten, and a
 * call returns when y holds the result.  Device memory is managed by the
 * library (grow-only per-device buffers reused across calls; the reference
 * allocates and frees per call).
 *
 * Differences (by design):
 *  - one GPU per process: ngpu must be 1, otherwise the call fails;
 *  - failures never exit the process (the reference's checkCudaErrors calls
 *    exit(EXIT_FAILURE), include/detail/cuda/helper_cuda.h:583-595): every
 *    spmv_ret field is -1 and sblas_last_error() holds the reason;
 *  - by default every entry point computes y = alpha*A*x + beta*y on all
 *    rows (README.md:118-119); sblas_set_compat_mode(1) reproduces the
 *    reference's ngpu = 1 results where they differ (see sblas_gb300.h).
 */
#ifndef SPMV_KERNEL
#define SPMV_KERNEL

#include <stddef.h>
#include "sblas_gb300.h"

#ifdef __cplusplus
#include <cstdio>
#include <sstream>
#include <string>
#include <iostream>
#endif

typedef struct CUstream_st *sblas_cuda_stream_t; /* same type as cudaStream_t */

/* include/spmv_kernel.h:16-57 -- per-phase seconds of one call */
struct spmv_ret {
    double numa_part_time;
    double part_time;
    double comp_time;
    double comm_time;
    double merg_time;
#ifdef __cplusplus
    void init() { numa_part_time = part_time = comp_time = comm_time = merg_time = 0.0; }
    void add(struct spmv_ret other)
    {
        numa_part_time += other.numa_part_time;
        part_time += other.part_time;
        comp_time += other.comp_time;
        comm_time += other.comm_time;
        merg_time += other.merg_time;
    }
    void avg(int n)
    {
        numa_part_time /= n;
        part_time /= n;
        comp_time /= n;
        comm_time /= n;
        merg_time /= n;
    }
    void print()
    {
        printf("%f, %f, %f, %f, %f\n", numa_part_time, part_time, comm_time, comp_time,
               merg_time);
    }
    std::string to_string()
    {
        std::ostringstream s;
        s << numa_part_time << "," << part_time << "," << comm_time << "," << comp_time << ","
          << merg_time << "\n";
        return s.str();
    }
#endif
};
#ifndef __cplusplus
typedef struct spmv_ret spmv_ret;
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* include/spmv_kernel.h:205-209 -- per-GPU kernel 3 wrapper; DEVICE arrays,
 * asynchronous on `stream` (a cudaStream_t).  Returns 0 or a status code. */
SBLAS_API int csr5_kernel(int m, int n, int nnz, double *alpha, double *csrVal, int *csrRowPtr,
                int *csrColIndex, double *x, double *beta, double *y,
                sblas_cuda_stream_t stream);

/* :211-215 */
SBLAS_API struct spmv_ret spMV_mgpu_baseline(int m, int n, int nnz, double *alpha, double *csrVal,
                                   int *csrRowPtr, int *csrColIndex, double *x, double *beta,
                                   double *y, int ngpu);
/* :217-221 */
SBLAS_API struct spmv_ret spMV_mgpu_baseline_csc(int m, int n, int nnz, double *alpha, double *cscVal,
                                       int *cscColPtr, int *cscRowIdx, double *x, double *beta,
                                       double *y, int ngpu);
/* :223-227 (COO sorted by row, as the reference requires) */
SBLAS_API struct spmv_ret spMV_mgpu_baseline_coo(int m, int n, int nnz, double *alpha, double *cooVal,
                                       int *cooRowIdx, int *cooColIdx, double *x, double *beta,
                                       double *y, int ngpu);
/* :229-234 */
SBLAS_API struct spmv_ret spMV_mgpu_v1(int m, int n, int nnz, double *alpha, double *csrVal,
                             int *csrRowPtr, int *csrColIndex, double *x, double *beta,
                             double *y, int ngpu, int kernel);
/* :236-244 */
SBLAS_API struct spmv_ret spMV_mgpu_v1_numa(int m, int n, int nnz, double *alpha, double *csrVal,
                                  int *csrRowPtr, int *csrColIndex, double *x, double *beta,
                                  double *y, int ngpu, int kernel, int *numa_mapping,
                                  int part_opt, int merg_opt);
/* :246-254 (nnz is long long in the reference's declaration) */
SBLAS_API struct spmv_ret spMV_mgpu_v1_numa_csc(int m, int n, long long nnz, double *alpha,
                                      double *cscVal, int *cscColPtr, int *cscRowIndex,
                                      double *x, double *beta, double *y, int ngpu, int kernel,
                                      int *numa_mapping, int part_opt, int merg_opt);
/* :256-264 */
SBLAS_API struct spmv_ret spMV_mgpu_v1_numa_coo(int m, int n, int nnz, double *alpha, double *cooVal,
                                      int *cooRowIdx, int *cooColIdx, double *x, double *beta,
                                      double *y, int ngpu, int kernel, int *numa_mapping,
                                      int part_opt, int merg_opt);
/* :266-273 */
SBLAS_API struct spmv_ret spMV_mgpu_v2(int m, int n, int nnz, double *alpha, double *csrVal,
                             int *csrRowPtr, int *csrColIndex, double *x, double *beta,
                             double *y, int ngpu, int kernel, int nb, int copy_of_workspace);
/* :276-296 -- SpMV restricted to the nonzeros whose x entry is nonzero */
SBLAS_API struct spmv_ret spMspV_mgpu_v1(int m, int n, int nnz, double *alpha, double *csrVal,
                               int *csrRowPtr, int *csrColIndex, double *x, double *beta,
                               double *y, int ngpu, int kernel);
SBLAS_API struct spmv_ret spMspV_mgpu_v2(int m, int n, int nnz, double *alpha, double *csrVal,
                               int *csrRowPtr, int *csrColIndex, double *x, double *beta,
                               double *y, int ngpu, int kernel, int nb, int copy_of_workspace);

/* helpers, :300-351 */
SBLAS_API int get_row_from_index(int n, int *a, int idx);
SBLAS_API double get_time(void);
SBLAS_API double get_gpu_availble_mem(int ngpu);
SBLAS_API void coo2csr(int m, int n, int nnz, double *cooVal, int *cooRowIdx, int *cooColIdx,
             double *csrVal, int *csrRowPtr, int *csrColIdx);
SBLAS_API void coo2csc(int m, int n, int nnz, double *cooVal, int *cooRowIdx, int *cooColIdx,
             double *cscVal, int *cscColPtr, int *cscRowIdx);
SBLAS_API void sortCOORow(int m, int n, int nnz, double *cooVal, int *cooRowIdx, int *cooColIdx);
SBLAS_API void sortCOOCol(int m, int n, int nnz, double *cooVal, int *cooRowIdx, int *cooColIdx);
/* device arrays; the handle argument (a cusparseHandle_t in the reference) is unused */
SBLAS_API void coo2csrGPU(void *handle, sblas_cuda_stream_t stream, int m, int n, int nnz,
                double *cooVal, int *cooRowIdx, int *cooColIdx, double *csrVal,
                int *csrRowPtr, int *csrColIdx);
SBLAS_API int findFirstInSorted(int *a, int n, int key);
SBLAS_API int findLastInSorted(int *a, int n, int key);
SBLAS_API void report_mem_usage(int d);
SBLAS_API void report_all_mem_usage(void);
SBLAS_API void print_vec_double(double *a, int n, const char *s);
SBLAS_API void print_vec_int(int *a, int n, const char *s);
SBLAS_API void print_vec_gpu_double(double *a, int n, const char *s);
SBLAS_API void print_vec_gpu_int(int *a, int n, const char *s);

#ifdef __cplusplus
}  /* extern "C" */

/* :11-14 -- C++ overloads of the print helpers */
inline void print_vec(double *a, int n, std::string s) { print_vec_double(a, n, s.c_str()); }
inline void print_vec(int *a, int n, std::string s) { print_vec_int(a, n, s.c_str()); }
inline void print_vec_gpu(double *a, int n, std::string s) { print_vec_gpu_double(a, n, s.c_str()); }
inline void print_vec_gpu(int *a, int n, std::string s) { print_vec_gpu_int(a, n, s.c_str()); }

/* :7 -- the reference's header includes common_cuda.h, which brings in the
 * CUDA samples' checkCudaErrors; the test programs wrap their own CUDA calls
 * (cudaGetDeviceCount, cudaMallocHost) in it.  This stand-in keeps them
 * compiling unchanged: a failing call (non-zero status) is reported with
 * its file, line and error number and ends the program, as there.  The
 * library's own entry points never exit (they return a status). */
#ifndef checkCudaErrors
#include <cstdlib>
template <typename Status>
inline void sblas_check_caller_cuda(Status rc, const char *call, const char *file, int line)
{
    if (static_cast<int>(rc) != 0) {
        std::fprintf(stderr, "%s:%d: %s failed with CUDA error %d\n", file, line, call,
                     static_cast<int>(rc));
        std::exit(EXIT_FAILURE);
    }
}
#define checkCudaErrors(call) sblas_check_caller_cuda((call), #call, __FILE__, __LINE__)
#endif
#endif

#endif /* SPMV_KERNEL */
