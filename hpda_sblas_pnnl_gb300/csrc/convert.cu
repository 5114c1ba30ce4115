// Format conversion on the device (setup work, not the SpMV hot path).
//
// The reference converts on the GPU with cuSPARSE: coo2csrGPU =
// cusparseXcoo2csr (src/spmv_helper.cu:478-490) after a stable row sort
// (sortCOORowGPU, :427-443); coo2csc = a stable column sort then the same
// compression with rows and columns swapped (:575-642).  Here, with this
// library's own kernels only:
//   * row-sorted COO -> CSR row pointer: atomic-free boundary detection (each
//     nonzero whose row differs from its left neighbour writes the row
//     pointer entries of the rows in between);
//   * sorts (CSC -> CSR, A -> A^T, the COO sorts): a stable least-significant-
//     digit sort by the row (or column) index, digits of at most 11 bits
//     (bucket_sort.cuh: per-tile digit counts, an exclusive scan, a stable
//     scatter): two passes for keys below 4M, three up to 2^31.  The first
//     pass derives what the entries carry from the source (a CSC entry's
//     column from the column pointer, an entry's own position), so no
//     permutation has to be applied afterwards; stability keeps the second
//     index ascending inside each row, as cuSPARSE's stable coosort does;
//   * spMspV's x-zero filter: a keep flag per nonzero, an exclusive scan of
//     the flags giving every kept nonzero its output position and every row
//     its new row pointer, then a scatter.
#include "bucket_sort.cuh"
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

int grid_for(long long items, int threads)
{
    const long long want = (items + threads - 1) / threads;
    const long long cap = 8LL * device_num_sms();
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
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

namespace {

// Buffers of one stable least-significant-digit sort of n entries: the pass
// scratch (digit-count table, scan sums) and, for two passes or more, one or
// two sets of intermediate arrays (key, a, b, d as present).
struct LsdLayout {
    size_t pass = 0, set = 0, total = 0;
    int passes = 0, width = 0;
};

LsdLayout lsd_layout(long long n, long long key_bound, bool has_a, bool has_b, bool has_d)
{
    LsdLayout L;
    const bsort::LsdPlan plan = bsort::lsd_plan(key_bound);
    L.passes = plan.passes;
    L.width = plan.width;
    const size_t nn = (size_t)(n > 0 ? n : 1);
    L.pass = al256(bsort::pass_work_bytes(n > 0 ? n : 1, 1 << plan.width));
    L.set = al256(4 * nn) + (has_a ? al256(4 * nn) : 0) + (has_b ? al256(4 * nn) : 0) +
            (has_d ? al256(8 * nn) : 0);
    L.total = L.pass + (size_t)(L.passes >= 3 ? 2 : (L.passes == 2 ? 1 : 0)) * L.set;
    return L;
}

struct ArraySet {
    int *key = nullptr, *a = nullptr, *b = nullptr;
    double *d = nullptr;
};

ArraySet array_set(unsigned char *p, long long n, bool has_a, bool has_b, bool has_d)
{
    const size_t nn = (size_t)(n > 0 ? n : 1);
    ArraySet s;
    s.key = reinterpret_cast<int *>(p);
    p += al256(4 * nn);
    if (has_a) {
        s.a = reinterpret_cast<int *>(p);
        p += al256(4 * nn);
    }
    if (has_b) {
        s.b = reinterpret_cast<int *>(p);
        p += al256(4 * nn);
    }
    if (has_d) s.d = reinterpret_cast<double *>(p);
    return s;
}

// Stable sort of n entries by key in [0, key_bound).  Pass 1 reads through
// `first` (its outputs are set here); later passes move the arrays; the last
// pass writes `out` (out.key required; out.a / out.b / out.d as the first
// operation carries them).
template <class FirstOp>
int lsd_sort(FirstOp first, long long n, long long key_bound, const ArraySet &out, void *work,
             size_t work_bytes, cudaStream_t stream)
{
    if (n <= 0) return SBLAS_OK;
    const bool has_a = out.a != nullptr, has_b = out.b != nullptr, has_d = out.d != nullptr;
    const LsdLayout L = lsd_layout(n, key_bound, has_a, has_b, has_d);
    if (work == nullptr || work_bytes < L.total) {
        set_error(SBLAS_ERR_ARG, "sort workspace too small (%zu < %zu)", work_bytes, L.total);
        return SBLAS_ERR_ARG;
    }
    unsigned char *w = static_cast<unsigned char *>(work);
    ArraySet tmp[2] = {array_set(w + L.pass, n, has_a, has_b, has_d),
                       array_set(w + L.pass + L.set, n, has_a, has_b, has_d)};
    const int nb = 1 << L.width;
    for (int p = 0; p < L.passes; ++p) {
        const ArraySet &dst = (p == L.passes - 1) ? out : tmp[p % 2];
        int rc;
        if (p == 0) {
            FirstOp op = first;
            op.key_out = dst.key;
            op.a_out = dst.a;
            op.b_out = dst.b;
            op.d_out = dst.d;
            rc = bsort::scatter_pass(op, n, 0, nb, w, stream);
        } else {
            const ArraySet &src = tmp[(p - 1) % 2];
            bsort::MoveOp op{src.key, src.a, src.b, src.d, dst.key, dst.a, dst.b, dst.d};
            rc = bsort::scatter_pass(op, n, p * L.width, nb, w, stream);
        }
        if (rc != SBLAS_OK) return rc;
    }
    return SBLAS_OK;
}

}  // namespace

size_t csc_to_csr_workspace_bytes(int m, int n, long long nnz)
{
    (void)n;
    const size_t nn = (size_t)(nnz > 0 ? nnz : 1);
    return al256(4 * nn) + lsd_layout(nnz, m, true, false, true).total;
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
    const size_t need = csc_to_csr_workspace_bytes(m, n, nnz);
    if (work == nullptr || work_bytes < need) {
        set_error(SBLAS_ERR_ARG, "csc_to_csr workspace too small (%zu < %zu)", work_bytes, need);
        return SBLAS_ERR_ARG;
    }
    unsigned char *w = static_cast<unsigned char *>(work);
    ArraySet out;
    out.key = reinterpret_cast<int *>(w);   // the rows, sorted: the row pointer's source
    out.a = csr_col;
    out.d = csr_val;
    // pass 1 reads the CSC arrays: key = row, a = column (from the column
    // pointer), d = value
    bsort::SegmentOp first{csc_row, csc_colptr, n, csc_val, nullptr, nullptr, nullptr, nullptr};
    const int rc = lsd_sort(first, nnz, m, out, w + al256(4 * (size_t)nnz),
                            work_bytes - al256(4 * (size_t)nnz), stream);
    if (rc != SBLAS_OK) return rc;
    return launch_coo_rows_to_rowptr(m, nnz, out.key, csr_rowptr, stream);
}

size_t coo_sort_workspace_bytes(int key_bound, long long nnz)
{
    return lsd_layout(nnz, key_bound, true, false, true).total;
}

int launch_coo_sort(int key_bound, long long nnz, const int *keys, const int *other,
                    const double *val, int *keys_out, int *other_out, double *val_out,
                    void *work, size_t work_bytes, cudaStream_t stream)
{
    if (nnz <= 0) return SBLAS_OK;
    ArraySet out;
    out.key = keys_out;
    out.a = other_out;
    out.d = val_out;
    bsort::MoveOp first{keys, other, nullptr, val, nullptr, nullptr, nullptr, nullptr};
    return lsd_sort(first, nnz, key_bound, out, work, work_bytes, stream);
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
    const size_t nn = (size_t)(nnz > 0 ? nnz : 1);
    return al256(4 * nn) + lsd_layout(nnz, n, true, true, false).total;
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
    const size_t need = csr_transpose_workspace_bytes(m, n, nnz);
    if (work == nullptr || work_bytes < need) {
        set_error(SBLAS_ERR_ARG, "csr_transpose workspace too small (%zu < %zu)", work_bytes, need);
        return SBLAS_ERR_ARG;
    }
    unsigned char *w = static_cast<unsigned char *>(work);
    ArraySet out;
    out.key = reinterpret_cast<int *>(w);   // the columns, sorted: A^T's row pointer source
    out.a = t_col;                          // the row of A holding the entry
    out.b = perm;                           // the entry's position in A
    // stable by column: the entries of one column keep their row order
    bsort::SegmentOp first{col, rowptr, m, nullptr, nullptr, nullptr, nullptr, nullptr};
    const int rc = lsd_sort(first, nnz, n, out, w + al256(4 * (size_t)nnz),
                            work_bytes - al256(4 * (size_t)nnz), stream);
    if (rc != SBLAS_OK) return rc;
    return launch_coo_rows_to_rowptr(n, nnz, out.key, t_rowptr, stream);
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

size_t filter_scan_bytes(long long nnz) { return bsort::scan_tmp_bytes(nnz + 1); }
}  // namespace

size_t csr_filter_x_workspace_bytes(long long nnz)
{
    if (nnz < 0) nnz = 0;
    return al256(filter_scan_bytes(nnz)) + 2 * al256(sizeof(int) * (size_t)(nnz + 1));
}

int launch_csr_filter_x(int m, long long nnz, const int *rowptr, const int *col,
                        const double *val, const double *x, int *orowptr, int *ocol,
                        double *oval, void *work, size_t work_bytes, cudaStream_t stream)
{
    if (m < 0 || nnz < 0 || nnz >= 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d nnz=%lld", m, nnz);
        return SBLAS_ERR_ARG;
    }
    const size_t scan_bytes = filter_scan_bytes(nnz);
    const size_t need = al256(scan_bytes) + 2 * al256(sizeof(int) * (size_t)(nnz + 1));
    if (work == nullptr || work_bytes < need) {
        set_error(SBLAS_ERR_ARG, "csr_filter_x workspace too small (%zu < %zu)", work_bytes, need);
        return SBLAS_ERR_ARG;
    }
    unsigned char *w = static_cast<unsigned char *>(work);
    int *flag = reinterpret_cast<int *>(w + al256(scan_bytes));
    int *pos = reinterpret_cast<int *>(w + al256(scan_bytes) + al256(sizeof(int) * (nnz + 1)));
    filter_flags_kernel<<<grid_for(nnz + 1, 256), 256, 0, stream>>>(nnz, col, x, flag);
    SBLAS_CUDA_TRY(cudaGetLastError());
    const int src = bsort::exclusive_scan(flag, pos, nnz + 1, w, nullptr, stream);
    if (src != SBLAS_OK) return src;
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
