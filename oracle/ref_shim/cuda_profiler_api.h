/* Host-only stand-in for <cuda_profiler_api.h>; see cuda_runtime.h here. */
#ifndef SBLAS_REF_SHIM_PROFILER_H
#define SBLAS_REF_SHIM_PROFILER_H
#include "cuda_runtime.h"
SBLAS_SHIM_STUB(cudaProfilerStart) SBLAS_SHIM_STUB(cudaProfilerStop)
#endif
