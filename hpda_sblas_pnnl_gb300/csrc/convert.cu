// Format conversion on the device (setup work, not the SpMV hot path).
//
// The reference converts on the GPU with cuSPARSE: coo2csrGPU =
// cusparseXcoo2csr (src/spmv_helper.cu:478-490) after a stable row sort
// (sortCOORowGPU, :427-443); coo2csc = a stable column sort then the same
// compression with rows and columns swapped (:575-642).  Here:
//   * row-sorted COO -> CSR row pointer: atomic-free boundary detection (each
//     nonzero whose row differs from its left neighbour writes the row
//     pointer entries of the rows in between);
//   * CSC -> CSR: a stable radix sort of (row, CSC position) pairs (CUB,
//     part of the CUDA toolkit), then a gather of column and value; stability
//     keeps columns ascending inside each row, as cuSPARSE's stable coosort;
//   * spMspV's x-zero filter: a keep flag per nonzero, an exclusive scan of
//     the flags (CUB) giving every kept nonzero its output position and every
//     row its new row pointer, then a scatter.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "sblas_internal.h"

namespace sblas {
namespace {

// Rows prev+1 .. cur start at nonzero k (nothing for an unsorted pair).  Row
// indices outside [0, m) never produce a write outside rowptr[0 .. m].
__device__ __forceinline__ void rows_start_at(int prev, int cur, int m, long long k,
                                              int *__restrict__ rowptr)
{
    for (int r = max(prev + 1, 0); r <= cur && r <= m; ++r) rowptr[r] = (int)k;
}

// One nonzero per thread (row arrays that are not 16-byte aligned); an index
// outside [0, m) or a decrease (unsorted input) writes nothing.
__global__ void coo_rowptr_kernel(int m, long long nnz, const int *__restrict__ row,
                                  int *__restrict__ rowptr)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k <= nnz; k += stride) {
        const int prev = (k == 0) ? -1 : __ldg(row + k - 1);
        const int cur = (k == nnz) ? m : __ldg(row + k);
        if ((k < nnz && (cur < 0 || cur >= m)) || cur < prev) continue;
        // rows prev+1 .. cur start at k (row `cur` itself starts at k too)
        rows_start_at(prev, cur, m, k, rowptr);
    }
}

// The same as coo_rowptr_kernel for a 16-byte aligned row array: every
// thread takes four consecutive nonzeros with one 16-byte load (four times
// the bytes in flight of the one-index form, which ran at about a quarter of
// HBM speed), the left neighbour of the first from the previous quad.
__global__ void coo_rowptr_quad_kernel(int m, long long nnz, const int *__restrict__ row,
                                       int *__restrict__ rowptr)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nq = nnz / 4;
    const int4 *q4 = reinterpret_cast<const int4 *>(row);
    auto quad = [&](const int4 v, int prev, long long k) {
        rows_start_at(prev, min(v.x, m - 1), m, k, rowptr);
        rows_start_at(v.x, min(v.y, m - 1), m, k + 1, rowptr);
        rows_start_at(v.y, min(v.z, m - 1), m, k + 2, rowptr);
        rows_start_at(v.z, min(v.w, m - 1), m, k + 3, rowptr);
    };
    // two quads per iteration, both loaded before either is used
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq;
         q += 2 * stride) {
        const long long q2 = q + stride;
        const bool two = q2 < nq;
        const int4 v = __ldg(q4 + q);
        const int4 w = two ? __ldg(q4 + q2) : v;
        const int pv = (q == 0) ? -1 : __ldg(row + 4 * q - 1);
        const int pw = two ? __ldg(row + 4 * q2 - 1) : 0;
        quad(v, pv, 4 * q);
        if (two) quad(w, pw, 4 * q2);
    }
    // the last nnz % 4 nonzeros and the end (rows after the last nonzero)
    for (long long k = 4 * nq + (long long)blockIdx.x * blockDim.x + threadIdx.x; k <= nnz;
         k += stride) {
        const int prev = (k == 0) ? -1 : __ldg(row + k - 1);
        const int cur = (k == nnz) ? m : min(__ldg(row + k), m - 1);
        rows_start_at(prev, cur, m, k, rowptr);
    }
}

__global__ void zero_rowptr_kernel(int m, int *rowptr)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= m; i += gridDim.x * blockDim.x)
        rowptr[i] = 0;
}

__global__ void iota_kernel(long long nnz, int *v)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
         k += (long long)gridDim.x * blockDim.x)
        v[k] = (int)k;
}

// CSC position k -> its column (largest j with colptr[j] <= k, skipping
// empty columns), then gather column and value into CSR order.
__global__ void csc_gather_kernel(int n, long long nnz, const int *__restrict__ colptr,
                                  const int *__restrict__ perm, const double *__restrict__ cval,
                                  int *__restrict__ ocol, double *__restrict__ oval)
{
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < nnz;
         p += (long long)gridDim.x * blockDim.x) {
        const int k = __ldg(perm + p);
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(colptr + mid) <= k) lo = mid; else hi = mid - 1;
        }
        ocol[p] = lo;
        oval[p] = __ldg(cval + k);
    }
}

int grid_for(long long items, int threads)
{
    const long long want = (items + threads - 1) / threads;
    const long long cap = 8LL * device_num_sms();
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

int end_bit_for(int m)
{
    int b = 1;
    while (b < 31 && (1LL << b) < (long long)m) ++b;
    return b;
}

size_t al256(size_t v) { return (v + 255) & ~size_t(255); }

}  // namespace

int launch_coo_rows_to_rowptr(int m, long long nnz, const int *coo_row, int *rowptr,
                              cudaStream_t stream)
{
    if (m < 0 || nnz < 0) {
        set_error(SBLAS_ERR_ARG, "negative size");
        return SBLAS_ERR_ARG;
    }
    if (nnz == 0) {
        zero_rowptr_kernel<<<grid_for((long long)m + 1, 256), 256, 0, stream>>>(m, rowptr);
    } else if ((reinterpret_cast<uintptr_t>(coo_row) & 15) == 0) {
        coo_rowptr_quad_kernel<<<grid_for(nnz / 4 + 1, 256), 256, 0, stream>>>(m, nnz, coo_row,
                                                                              rowptr);
    } else {
        coo_rowptr_kernel<<<grid_for(nnz + 1, 256), 256, 0, stream>>>(m, nnz, coo_row, rowptr);
    }
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

size_t csc_to_csr_workspace_bytes(int m, int n, long long nnz)
{
    (void)n;
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs<int, int>(nullptr, cub_bytes, (const int *)nullptr,
                                              (int *)nullptr, (const int *)nullptr,
                                              (int *)nullptr, (int)nnz, 0, end_bit_for(m));
    return al256(cub_bytes) + 3 * al256(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
}

int launch_csc_to_csr(int m, int n, long long nnz, const double *csc_val, const int *csc_colptr,
                      const int *csc_row, double *csr_val, int *csr_rowptr, int *csr_col,
                      void *work, size_t work_bytes, cudaStream_t stream)
{
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d n=%d nnz=%lld", m, n, nnz);
        return SBLAS_ERR_ARG;
    }
    if (nnz == 0) return launch_coo_rows_to_rowptr(m, 0, nullptr, csr_rowptr, stream);
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs<int, int>(nullptr, cub_bytes, (const int *)nullptr,
                                              (int *)nullptr, (const int *)nullptr,
                                              (int *)nullptr, (int)nnz, 0, end_bit_for(m));
    const size_t need = al256(cub_bytes) + 3 * al256(sizeof(int) * (size_t)nnz);
    if (work == nullptr || work_bytes < need) {
        set_error(SBLAS_ERR_ARG, "csc_to_csr workspace too small (%zu < %zu)", work_bytes, need);
        return SBLAS_ERR_ARG;
    }
    unsigned char *w = static_cast<unsigned char *>(work);
    void *cub_tmp = w;
    int *perm_in = reinterpret_cast<int *>(w + al256(cub_bytes));
    int *perm_out = reinterpret_cast<int *>(w + al256(cub_bytes) + al256(sizeof(int) * nnz));
    int *rows_sorted =
        reinterpret_cast<int *>(w + al256(cub_bytes) + 2 * al256(sizeof(int) * nnz));
    iota_kernel<<<grid_for(nnz, 256), 256, 0, stream>>>(nnz, perm_in);
    SBLAS_CUDA_TRY(cudaGetLastError());
    SBLAS_CUDA_TRY((cub::DeviceRadixSort::SortPairs<int, int>(cub_tmp, cub_bytes, csc_row,
                                                              rows_sorted, perm_in, perm_out,
                                                              (int)nnz, 0, end_bit_for(m),
                                                              stream)));
    csc_gather_kernel<<<grid_for(nnz, 256), 256, 0, stream>>>(n, nnz, csc_colptr, perm_out,
                                                              csc_val, csr_col, csr_val);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return launch_coo_rows_to_rowptr(m, nnz, rows_sorted, csr_rowptr, stream);
}

size_t sort_perm_workspace_bytes(int key_bound, long long nnz)
{
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs<int, int>(nullptr, cub_bytes, (const int *)nullptr,
                                              (int *)nullptr, (const int *)nullptr,
                                              (int *)nullptr, (int)nnz, 0, end_bit_for(key_bound));
    return al256(cub_bytes) + al256(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
}

int launch_sort_perm(int key_bound, long long nnz, const int *keys, int *keys_sorted, int *perm,
                     void *work, size_t work_bytes, cudaStream_t stream)
{
    if (nnz <= 0) return SBLAS_OK;
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs<int, int>(nullptr, cub_bytes, (const int *)nullptr,
                                              (int *)nullptr, (const int *)nullptr,
                                              (int *)nullptr, (int)nnz, 0, end_bit_for(key_bound));
    if (work_bytes < al256(cub_bytes) + al256(sizeof(int) * (size_t)nnz)) {
        set_error(SBLAS_ERR_ARG, "sort workspace too small");
        return SBLAS_ERR_ARG;
    }
    unsigned char *w = static_cast<unsigned char *>(work);
    int *iota = reinterpret_cast<int *>(w + al256(cub_bytes));
    iota_kernel<<<grid_for(nnz, 256), 256, 0, stream>>>(nnz, iota);
    SBLAS_CUDA_TRY(cudaGetLastError());
    SBLAS_CUDA_TRY((cub::DeviceRadixSort::SortPairs<int, int>(w, cub_bytes, keys, keys_sorted, iota,
                                                              perm, (int)nnz, 0,
                                                              end_bit_for(key_bound), stream)));
    return SBLAS_OK;
}

namespace {
__global__ void gather_kernel(long long nnz, const int *__restrict__ perm,
                              const int *__restrict__ in_i, int *__restrict__ out_i,
                              const double *__restrict__ in_d, double *__restrict__ out_d)
{
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < nnz;
         p += (long long)gridDim.x * blockDim.x) {
        const int k = __ldg(perm + p);
        if (out_i) out_i[p] = __ldg(in_i + k);
        if (out_d) out_d[p] = __ldg(in_d + k);
    }
}
}  // namespace

namespace {
// Entry q of A^T is entry perm[q] of A: its column in A^T is the row of A
// holding position perm[q] (largest r with rowptr[r] <= perm[q]).
__global__ void transpose_rows_kernel(int m, long long nnz, const int *__restrict__ rowptr,
                                      const int *__restrict__ perm, int *__restrict__ t_col)
{
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nnz;
         q += (long long)gridDim.x * blockDim.x) {
        const int p = __ldg(perm + q);
        int lo = 0, hi = m - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(rowptr + mid) <= p) lo = mid; else hi = mid - 1;
        }
        t_col[q] = lo;
    }
}

__global__ void gather_f32_kernel(long long nnz, const int *__restrict__ perm,
                                  const float *__restrict__ in, float *__restrict__ out)
{
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < nnz;
         p += (long long)gridDim.x * blockDim.x)
        out[p] = __ldg(in + __ldg(perm + p));
}
}  // namespace

size_t csr_transpose_workspace_bytes(int m, int n, long long nnz)
{
    (void)m;
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs<int, int>(nullptr, cub_bytes, (const int *)nullptr,
                                              (int *)nullptr, (const int *)nullptr,
                                              (int *)nullptr, (int)nnz, 0, end_bit_for(n));
    return al256(cub_bytes) + 2 * al256(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
}

int launch_csr_transpose(int m, int n, long long nnz, const int *rowptr, const int *col,
                         int *t_rowptr, int *t_col, int *perm, void *work, size_t work_bytes,
                         cudaStream_t stream)
{
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d n=%d nnz=%lld", m, n, nnz);
        return SBLAS_ERR_ARG;
    }
    if (nnz == 0) return launch_coo_rows_to_rowptr(n, 0, nullptr, t_rowptr, stream);
    size_t cub_bytes = 0;
    cub::DeviceRadixSort::SortPairs<int, int>(nullptr, cub_bytes, (const int *)nullptr,
                                              (int *)nullptr, (const int *)nullptr,
                                              (int *)nullptr, (int)nnz, 0, end_bit_for(n));
    const size_t need = al256(cub_bytes) + 2 * al256(sizeof(int) * (size_t)nnz);
    if (work == nullptr || work_bytes < need) {
        set_error(SBLAS_ERR_ARG, "csr_transpose workspace too small (%zu < %zu)", work_bytes, need);
        return SBLAS_ERR_ARG;
    }
    unsigned char *w = static_cast<unsigned char *>(work);
    int *iota = reinterpret_cast<int *>(w + al256(cub_bytes));
    int *cols_sorted = reinterpret_cast<int *>(w + al256(cub_bytes) + al256(sizeof(int) * nnz));
    iota_kernel<<<grid_for(nnz, 256), 256, 0, stream>>>(nnz, iota);
    SBLAS_CUDA_TRY(cudaGetLastError());
    // stable sort by column: entries of one column keep their row order
    SBLAS_CUDA_TRY((cub::DeviceRadixSort::SortPairs<int, int>(w, cub_bytes, col, cols_sorted, iota,
                                                              perm, (int)nnz, 0, end_bit_for(n),
                                                              stream)));
    transpose_rows_kernel<<<grid_for(nnz, 256), 256, 0, stream>>>(m, nnz, rowptr, perm, t_col);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return launch_coo_rows_to_rowptr(n, nnz, cols_sorted, t_rowptr, stream);
}

int launch_gather_values(long long nnz, int val_kind, const void *src, const int *perm, void *dst,
                         cudaStream_t stream)
{
    if (nnz <= 0) return SBLAS_OK;
    if (val_kind == VAL_F64)
        return launch_gather(nnz, perm, nullptr, nullptr, static_cast<const double *>(src),
                             static_cast<double *>(dst), stream);
    if (val_kind != VAL_F32) {
        set_error(SBLAS_ERR_ARG, "values of kind %d cannot be gathered", val_kind);
        return SBLAS_ERR_ARG;
    }
    gather_f32_kernel<<<grid_for(nnz, 256), 256, 0, stream>>>(nnz, perm,
                                                               static_cast<const float *>(src),
                                                               static_cast<float *>(dst));
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

int launch_gather(long long nnz, const int *perm, const int *in_i, int *out_i,
                  const double *in_d, double *out_d, cudaStream_t stream)
{
    if (nnz <= 0) return SBLAS_OK;
    gather_kernel<<<grid_for(nnz, 256), 256, 0, stream>>>(nnz, perm, in_i, out_i, in_d, out_d);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

namespace {
__global__ void filter_flags_kernel(long long nnz, const int *__restrict__ col,
                                    const double *__restrict__ x, int *__restrict__ flag)
{
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j <= nnz;
         j += (long long)gridDim.x * blockDim.x)
        flag[j] = (j < nnz && __ldg(x + __ldg(col + j)) != 0.0) ? 1 : 0;
}

__global__ void filter_scatter_kernel(long long nnz, const int *__restrict__ col,
                                      const double *__restrict__ val,
                                      const int *__restrict__ flag, const int *__restrict__ pos,
                                      int *__restrict__ ocol, double *__restrict__ oval)
{
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nnz;
         j += (long long)gridDim.x * blockDim.x)
        if (flag[j]) {
            const int q = pos[j];
            ocol[q] = __ldg(col + j);
            if (val) oval[q] = __ldg(val + j);
        }
}

__global__ void filter_rowptr_kernel(int m, const int *__restrict__ rowptr,
                                     const int *__restrict__ pos, int *__restrict__ orowptr)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i <= m;
         i += (long long)gridDim.x * blockDim.x)
        orowptr[i] = pos[__ldg(rowptr + i)];
}

size_t filter_cub_bytes(long long nnz)
{
    size_t cub_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, cub_bytes, (const int *)nullptr, (int *)nullptr,
                                  (int)(nnz + 1));
    return cub_bytes;
}
}  // namespace

size_t csr_filter_x_workspace_bytes(long long nnz)
{
    if (nnz < 0) nnz = 0;
    return al256(filter_cub_bytes(nnz)) + 2 * al256(sizeof(int) * (size_t)(nnz + 1));
}

int launch_csr_filter_x(int m, long long nnz, const int *rowptr, const int *col,
                        const double *val, const double *x, int *orowptr, int *ocol,
                        double *oval, void *work, size_t work_bytes, cudaStream_t stream)
{
    if (m < 0 || nnz < 0 || nnz >= 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d nnz=%lld", m, nnz);
        return SBLAS_ERR_ARG;
    }
    const size_t cub_bytes = filter_cub_bytes(nnz);
    const size_t need = al256(cub_bytes) + 2 * al256(sizeof(int) * (size_t)(nnz + 1));
    if (work == nullptr || work_bytes < need) {
        set_error(SBLAS_ERR_ARG, "csr_filter_x workspace too small (%zu < %zu)", work_bytes, need);
        return SBLAS_ERR_ARG;
    }
    unsigned char *w = static_cast<unsigned char *>(work);
    int *flag = reinterpret_cast<int *>(w + al256(cub_bytes));
    int *pos = reinterpret_cast<int *>(w + al256(cub_bytes) + al256(sizeof(int) * (nnz + 1)));
    filter_flags_kernel<<<grid_for(nnz + 1, 256), 256, 0, stream>>>(nnz, col, x, flag);
    SBLAS_CUDA_TRY(cudaGetLastError());
    size_t cb = cub_bytes;
    SBLAS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(w, cb, flag, pos, (int)(nnz + 1), stream));
    if (nnz > 0) {
        filter_scatter_kernel<<<grid_for(nnz, 256), 256, 0, stream>>>(nnz, col, val, flag, pos,
                                                                      ocol, oval);
        SBLAS_CUDA_TRY(cudaGetLastError());
    }
    filter_rowptr_kernel<<<grid_for((long long)m + 1, 256), 256, 0, stream>>>(m, rowptr, pos,
                                                                             orowptr);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

}  // namespace sblas
