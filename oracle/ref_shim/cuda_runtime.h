/* Host-only stand-in for <cuda_runtime.h>, used only to compile the
 * reference's CPU functions (csr_spmv_cpu, coo_spmv_cpu, get_row_from_index,
 * findFirst/LastInSorted) from its own sources with g++.  Every CUDA call in
 * those files becomes an inline stub that reports failure; none is called. */
#ifndef SBLAS_REF_SHIM_CUDA_RUNTIME_H
#define SBLAS_REF_SHIM_CUDA_RUNTIME_H
#include <cstddef>
typedef int cudaError_t;
typedef struct sblas_shim_stream *cudaStream_t;
typedef struct sblas_shim_event *cudaEvent_t;
typedef unsigned long long cudaTextureObject_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
                      cudaMemcpyDeviceToDevice, cudaMemcpyDefault };
struct cudaDeviceProp { char name[256]; int major, minor; };
#define SBLAS_SHIM_STUB(name) template <typename... A> static inline cudaError_t name(A &&...) { return 1; }
SBLAS_SHIM_STUB(cudaMalloc) SBLAS_SHIM_STUB(cudaMallocHost) SBLAS_SHIM_STUB(cudaFree)
SBLAS_SHIM_STUB(cudaFreeHost) SBLAS_SHIM_STUB(cudaMemcpy) SBLAS_SHIM_STUB(cudaMemcpyAsync)
SBLAS_SHIM_STUB(cudaSetDevice) SBLAS_SHIM_STUB(cudaGetDeviceCount) SBLAS_SHIM_STUB(cudaDeviceSynchronize)
SBLAS_SHIM_STUB(cudaStreamCreate) SBLAS_SHIM_STUB(cudaStreamDestroy) SBLAS_SHIM_STUB(cudaStreamSynchronize)
SBLAS_SHIM_STUB(cudaEventCreate) SBLAS_SHIM_STUB(cudaEventRecord) SBLAS_SHIM_STUB(cudaEventSynchronize)
SBLAS_SHIM_STUB(cudaEventElapsedTime) SBLAS_SHIM_STUB(cudaEventDestroy) SBLAS_SHIM_STUB(cudaMemGetInfo)
SBLAS_SHIM_STUB(cudaGetDeviceProperties) SBLAS_SHIM_STUB(cudaMemset)
static inline const char *cudaGetErrorString(cudaError_t) { return "shim"; }
#endif
