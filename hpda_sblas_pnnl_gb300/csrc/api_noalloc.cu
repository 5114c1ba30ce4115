// sblas_dcsrmv_noalloc: the FP64 CSR tile SpMV without any device allocation.
//
// Who needs it: code that cannot call cudaMalloc at the moment it needs an
// SpMV.  Typical cases are a caching allocator or memory pool that calls
// back into numerical code (a cudaMalloc there would re-enter the allocator
// or escape its budget), and services that reserve all device memory at
// start-up and forbid allocation afterwards (memory-capped or real-time
// loops).  sblas_dcsrmv needs either a caller-provided workspace or, with
// work = NULL, grows a library buffer with cudaMalloc; this entry point
// needs neither.
//
// Its scratch (the tile partition, the per-tile carries and a status word)
// lives in a file-scope __device__ array of fixed size, which every GPU that
// loads this library holds until the process exits.  Matrices whose scratch
// would exceed it are rejected with SBLAS_ERR_ARG.  Every call shares the
// array: calls that overlap on the GPU (different streams, or a stream not
// ordered after the previous call) race on it and must not be issued.  The
// scratch needs no clearing between calls: each call rewrites the partition
// and every carry it reads, and zeroes the status word with a memset node.
//
// Set-up: the first call on a device (with that device current) resolves the
// array's device address with cudaGetSymbolAddress and creates the
// library's per-device context (a CUDA stream and events), and configures the
// kernels the calls launch (loading them).  Under CUDA's
// default lazy module loading that first call is also when the library's
// module is loaded onto the device, and with it when the 7 MiB array gets
// its device memory; with CUDA_MODULE_LOADING=EAGER the array is placed when
// the library is loaded instead.  A call with m = 0 does the set-up and
// nothing else: make one before entering a region where allocation is
// forbidden, and before any stream capture.
//
// Failure detection: the kernels' bounded waits write the status word inside
// the array and the library's sticky device word; sblas_stream_status
// reports a wait that gave up.
#include <mutex>

#include "sblas_internal.h"

namespace sblas {
namespace {

constexpr size_t kNoallocScratchBytes = size_t(7) << 20;  // 7 MiB: ~0.86 G nonzeros at sigma 11
constexpr int kMaxDev = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDev] = {};

// Device address of g_noalloc_scratch on the current device (the host-side
// name of the array is only a stand-in, never a device address).
int noalloc_scratch(void **out)
{
    int dev = 0;
    SBLAS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDev) {
        set_error(SBLAS_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
        return SBLAS_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr) {
        void *p = nullptr;
        SBLAS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        if (p == nullptr) {
            set_error(SBLAS_ERR_CUDA, "cudaGetSymbolAddress returned a null scratch address");
            return SBLAS_ERR_CUDA;
        }
        if (device_context() == nullptr) {
            set_error(SBLAS_ERR_CUDA, "cannot create the per-device context");
            return SBLAS_ERR_CUDA;
        }
        // load every kernel the calls launch now, not at the first real call
        const int rc = tile_preload_f64(default_sigma_for(0, 0));
        if (rc != SBLAS_OK) return rc;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return SBLAS_OK;
}

}  // namespace
}  // namespace sblas

using namespace sblas;

extern "C" {

size_t sblas_noalloc_scratch_bytes(void) { return kNoallocScratchBytes; }

int sblas_dcsrmv_noalloc(int m, int n, int nnz, double alpha, const double *val,
                         const int *rowptr, const int *col, const double *x, double beta,
                         double *y, void *stream)
{
    clear_error();
    if (m < 0 || n < 0 || nnz < 0) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d n=%d nnz=%d", m, n, nnz);
        return SBLAS_ERR_ARG;
    }
    void *scratch = nullptr;
    const int rc = noalloc_scratch(&scratch);   // set-up on first use (m = 0: set-up only)
    if (rc != SBLAS_OK) return rc;
    if (m == 0) return SBLAS_OK;
    if (y == nullptr || (nnz > 0 && (val == nullptr || rowptr == nullptr || col == nullptr ||
                                     x == nullptr))) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    const int sigma = default_sigma_for(m, nnz);
    const size_t need = tile_workspace_bytes(nnz, sigma);
    if (need > kNoallocScratchBytes) {
        set_error(SBLAS_ERR_ARG,
                  "sblas_dcsrmv_noalloc: nnz=%d needs %zu bytes of scratch, more than its "
                  "static %zu bytes; use sblas_dcsrmv with a workspace",
                  nnz, need, kNoallocScratchBytes);
        return SBLAS_ERR_ARG;
    }
    return launch_tile_spmv(m, n, nnz, alpha, val, SBLAS_VAL_F64, rowptr, col, x, beta, y, sigma,
                            scratch, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
