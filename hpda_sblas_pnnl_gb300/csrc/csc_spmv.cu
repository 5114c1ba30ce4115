// y = alpha*A*x + beta*y with A in CSC: atomic-free and deterministic.
//
// The reference runs its CSC entry points as a transposed cuSPARSE csrmv
// (src/dspmv_mgpu_baseline_csc.cu:131-135), 4-33x slower than its CSR path.
// Here the work is split into an inspector, once per sparsity pattern, and
// an executor, once per product:
//   inspector  the row-ordered structure of A: a stable least-significant-
//              digit bucket sort of the CSC entries by row (bucket_sort.cuh)
//              carrying each entry's column and CSC position, giving A's CSR
//              row pointer, columns and the permutation perm (CSR position ->
//              CSC position), then the tile partition of that row pointer;
//   executor   the values in row order (one gather through perm, coalesced
//              writes) and the CSR tile kernel: its segmented sums and carry
//              fix-up in a fixed order, no atomics, bit-reproducible.
// sblas_dcscmv runs both; sblas_csc_analyse / sblas_dcscmv_analysed split
// them for a pattern used many times (the executor then costs one value
// gather, a random read of every value, more than a CSR product), and
// sblas_csc_bind_values keeps one set of values in row order inside the
// analysis, so that products with those values cost a CSR product alone.
#include "sblas_internal.h"

namespace sblas {
namespace {

size_t al256(size_t v) { return (v + 255) & ~size_t(255); }

constexpr int kCscSigma = 11;   // tile shape of the executor (the library default)

// Workspace: rowptr | col | perm | val (row order) | tile workspace | sort scratch
struct CscLayout {
    size_t rowptr, col, perm, val, tile, sort, total;
};

CscLayout csc_layout(int m, int n, long long nnz)
{
    const size_t nn = (size_t)(nnz > 0 ? nnz : 1);
    CscLayout L;
    L.rowptr = 0;
    L.col = L.rowptr + al256(4 * ((size_t)m + 1));
    L.perm = L.col + al256(4 * nn);
    L.val = L.perm + al256(4 * nn);
    L.tile = L.val + al256(8 * nn);
    L.sort = L.tile + al256(tile_workspace_bytes(nnz, kCscSigma));
    L.total = L.sort + al256(csr_transpose_workspace_bytes(n, m, nnz));
    return L;
}

// out[q] = val[perm[q]]: random reads of val (it does not fit in L2), so
// every thread keeps GATHER_ILP of them in flight: a stride of the grid
// between a thread's entries keeps each of its perm loads and out stores
// coalesced across the warp.
constexpr int GATHER_ILP = 8;

__global__ void __launch_bounds__(256) gather_rows_kernel(long long nnz,
                                                          const int *__restrict__ perm,
                                                          const double *__restrict__ val,
                                                          double *__restrict__ out)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; q0 < nnz;
         q0 += stride * GATHER_ILP) {
        int p[GATHER_ILP];
        double v[GATHER_ILP];
#pragma unroll
        for (int k = 0; k < GATHER_ILP; ++k) {
            const long long q = q0 + k * stride;
            p[k] = q < nnz ? __ldg(perm + q) : 0;
        }
#pragma unroll
        for (int k = 0; k < GATHER_ILP; ++k)
            v[k] = (q0 + k * stride < nnz) ? __ldg(val + p[k]) : 0.0;
#pragma unroll
        for (int k = 0; k < GATHER_ILP; ++k)
            if (q0 + k * stride < nnz) out[q0 + k * stride] = v[k];
    }
}

bool check_work(int m, int n, long long nnz, void *work, size_t work_bytes)
{
    const size_t need = csc_layout(m, n, nnz).total;
    if (work == nullptr || work_bytes < need || (reinterpret_cast<uintptr_t>(work) & 255) != 0) {
        set_error(SBLAS_ERR_ARG, "CSC SpMV workspace needs %zu bytes at 256-byte alignment",
                  need);
        return false;
    }
    return true;
}

}  // namespace

size_t cscmv_workspace_bytes(int m, int n, long long nnz) { return csc_layout(m, n, nnz).total; }

int launch_csc_analyse(int m, int n, long long nnz, const int *colptr, const int *rowidx,
                       void *work, size_t work_bytes, cudaStream_t stream)
{
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d n=%d nnz=%lld", m, n, nnz);
        return SBLAS_ERR_ARG;
    }
    if (m == 0 || nnz == 0) return SBLAS_OK;
    if (!check_work(m, n, nnz, work, work_bytes)) return SBLAS_ERR_ARG;
    const CscLayout L = csc_layout(m, n, nnz);
    unsigned char *w = static_cast<unsigned char *>(work);
    int *rowptr = reinterpret_cast<int *>(w + L.rowptr);
    // the CSC arrays are the CSR arrays of A^T (n rows): its transpose is A
    // in CSR, with every entry's CSC position as the permutation
    int rc = launch_csr_transpose(n, m, nnz, colptr, rowidx, rowptr,
                                  reinterpret_cast<int *>(w + L.col),
                                  reinterpret_cast<int *>(w + L.perm), w + L.sort,
                                  L.total - L.sort, stream);
    if (rc != SBLAS_OK) return rc;
    return launch_tile_analyse(m, nnz, rowptr, kCscSigma, w + L.tile, stream);
}

int launch_csc_bind_values(int m, int n, long long nnz, const double *val, void *work,
                           size_t work_bytes, cudaStream_t stream)
{
    if (m <= 0 || nnz <= 0) return SBLAS_OK;
    if (!check_work(m, n, nnz, work, work_bytes)) return SBLAS_ERR_ARG;
    const CscLayout L = csc_layout(m, n, nnz);
    unsigned char *w = static_cast<unsigned char *>(work);
    const long long want = (nnz + 255) / 256, cap = 16LL * device_num_sms();
    gather_rows_kernel<<<(unsigned)(want < cap ? want : cap), 256, 0, stream>>>(
        nnz, reinterpret_cast<const int *>(w + L.perm), val, reinterpret_cast<double *>(w + L.val));
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

int launch_cscmv_analysed(int m, int n, long long nnz, double alpha, const double *val,
                          const double *x, double beta, double *y, void *work,
                          size_t work_bytes, cudaStream_t stream)
{
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d n=%d nnz=%lld", m, n, nnz);
        return SBLAS_ERR_ARG;
    }
    if (m == 0) return SBLAS_OK;
    if (nnz == 0 || n == 0) return launch_scale_y(m, beta, y, stream);
    if (!check_work(m, n, nnz, work, work_bytes)) return SBLAS_ERR_ARG;
    const CscLayout L = csc_layout(m, n, nnz);
    unsigned char *w = static_cast<unsigned char *>(work);
    double *rval = reinterpret_cast<double *>(w + L.val);
    if (val != nullptr) {   // new values: into row order (else the bound ones)
        const int rc = launch_csc_bind_values(m, n, nnz, val, work, work_bytes, stream);
        if (rc != SBLAS_OK) return rc;
    }
    return launch_tile_spmv(m, n, nnz, alpha, rval, VAL_F64,
                            reinterpret_cast<const int *>(w + L.rowptr),
                            reinterpret_cast<const int *>(w + L.col), x, beta, y, kCscSigma,
                            w + L.tile, stream, true);
}

int launch_cscmv(int m, int n, long long nnz, double alpha, const double *val,
                 const int *colptr, const int *rowidx, const double *x, double beta, double *y,
                 void *work, size_t work_bytes, cudaStream_t stream)
{
    const int rc = launch_csc_analyse(m, n, nnz, colptr, rowidx, work, work_bytes, stream);
    if (rc != SBLAS_OK) return rc;
    return launch_cscmv_analysed(m, n, nnz, alpha, val, x, beta, y, work, work_bytes, stream);
}

void *csc_tile_workspace(void *work, int m, int n, long long nnz)
{
    return static_cast<unsigned char *>(work) + csc_layout(m, n, nnz).tile;
}

}  // namespace sblas
