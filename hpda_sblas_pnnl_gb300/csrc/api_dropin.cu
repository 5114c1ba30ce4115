// Drop-in entry points with the reference's signatures (include/spmv_kernel.h).
//
// Each entry point is the ngpu = 1 case of the reference function it
// replaces: partition (trivial for one part), host->device copies, one
// device kernel, device->host copy of y, merge.  Timing fields of spmv_ret
// follow the reference: comm_time = host->device copies (CUDA events,
// src/dspmv_mgpu_baseline.cu:114-120), comp_time = SpMV kernel (events,
// :124-130), part_time = partition / format work, merg_time = device->host
// copy and host merge (wall clock, :156-165), numa_part_time = 0 (no NUMA
// staging copy on a one-GPU, one-NUMA-node process).
#include <sys/time.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/spmv_kernel.h"
#include "sblas_internal.h"

namespace sblas {
namespace {

std::mutex g_dropin_mu;  // device buffers of the drop-in path are shared per process

spmv_ret failed()
{
    spmv_ret r;
    r.numa_part_time = r.part_time = r.comp_time = r.comm_time = r.merg_time = -1.0;
    return r;
}

spmv_ret zero_ret()
{
    spmv_ret r;
    r.numa_part_time = r.part_time = r.comp_time = r.comm_time = r.merg_time = 0.0;
    return r;
}

double wall()
{
    struct timeval tp;
    gettimeofday(&tp, nullptr);
    return (double)tp.tv_sec + (double)tp.tv_usec * 1e-6;
}

// src/spmv_helper.cu:18-44 restated: binary search over a[0..n]; the row that
// holds nonzero idx (skipping empty rows).
int row_of_index(int n, const int *a, int idx)
{
    int l = 0, r = n;
    while (l < r - 1) {
        const int mid = l + (r - l) / 2;
        if (idx < a[mid]) r = mid;
        else l = mid;
    }
    if (idx == a[l]) return l;
    if (idx == a[r]) return r;
    return l;
}

enum class Fmt { CSR, CSC, COO };

struct Call {
    const char *name;
    Fmt fmt;
    int m, n;
    long long nnz;
    double alpha, beta;
    const double *val;
    const int *ptr;   // CSR rowptr / CSC colptr / COO row index
    const int *idx;   // CSR col / CSC row / COO col
    const double *x;
    double *y;
    int kernel;       // 1, 2, 3
    int row_lo, row_hi;  // rows written: [row_lo, row_hi)
    bool additive;    // y_out = y0 + (alpha*A*x + beta*y0) on written rows
};

#define DROPIN_CUDA(expr)                                                                  \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            set_error(SBLAS_ERR_CUDA, "%s: %s failed: %s", c.name, #expr,                  \
                      cudaGetErrorString(e_));                                             \
            return failed();                                                               \
        }                                                                                  \
    } while (0)

bool check_common(const char *name, int m, int n, long long nnz, const double *alpha,
                  const double *beta, const void *val, const void *ptr, const void *idx,
                  const double *x, const double *y, int ngpu)
{
    if (ngpu != 1) {
        set_error(SBLAS_ERR_NGPU, "%s: ngpu=%d; this library drives one GPU per process (ngpu=1)",
                  name, ngpu);
        return false;
    }
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "%s: bad sizes m=%d n=%d nnz=%lld", name, m, n, nnz);
        return false;
    }
    if (!alpha || !beta) {
        set_error(SBLAS_ERR_ARG, "%s: alpha and beta must be non-null", name);
        return false;
    }
    if (m > 0 && !y) {
        set_error(SBLAS_ERR_ARG, "%s: y is null", name);
        return false;
    }
    if (nnz > 0 && (!val || !idx || !x)) {
        set_error(SBLAS_ERR_ARG, "%s: null matrix or x pointer", name);
        return false;
    }
    if ((m > 0 || nnz > 0) && !ptr) {
        set_error(SBLAS_ERR_ARG, "%s: null pointer array", name);
        return false;
    }
    return true;
}

bool check_kernel(const char *name, int kernel)
{
    if (kernel < 1 || kernel > 3) {
        set_error(SBLAS_ERR_ARG, "%s: kernel must be 1, 2 or 3 (got %d)", name, kernel);
        return false;
    }
    return true;
}

// Row pointer of one chunk rebased to its first nonzero: out[i] = rp[i] - base.
__global__ void rebase_rowptr_kernel(int count, const int *__restrict__ rp, int base, int *out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        out[i] = rp[i] - base;
}

constexpr long long kPipeMinNnz = 1LL << 22;   // smaller matrices: copy, then compute

// After the call's stream has completed: false (with SBLAS_ERR_TIMEOUT set)
// if a tile launch on workspace w gave up one of its bounded waits, which
// leaves y partly written.
bool launches_completed(const Call &c, void *w)
{
    int word = 0;
    if (tile_workspace_status(w, &word) != SBLAS_OK) return false;
    if (word != 0) {
        set_error(SBLAS_ERR_TIMEOUT, "%s: the SpMV kernel gave up a bounded wait (device word "
                  "%d); y is not valid", c.name, word);
        return false;
    }
    return true;
}

// Large CSR calls with host arrays: the matrix travels in kPipeChunks row
// chunks of equal nonzero counts, each chunk's SpMV starting as soon as its
// values and columns have arrived (copies on the context's copy stream, the
// tile kernel on its compute stream, y of a chunk sent back right after its
// kernel), so the kernels and the device-to-host copies hide behind the
// host-to-device copies, which the host link bounds.  Each chunk's arrays
// are placed at 256-byte aligned offsets so the tile kernel keeps its bulk
// copies; its row pointer is rebased to the chunk's first nonzero.
spmv_ret run_host_pipelined(const Call &c, DeviceContext *ctx)
{
    const int m = c.m, n = c.n;
    const long long nnz = c.nnz;
    const int K = kPipeChunks;
    const bool need_y_in = (c.beta != 0.0) || c.additive;
    cudaStream_t cs = ctx->copy_stream, ks = ctx->stream;
    // chunk k: rows [r[k], r[k+1]), nonzeros [ptr[r[k]], ptr[r[k+1]])
    int r[kPipeChunks + 1];
    r[0] = 0;
    r[K] = m;
    for (int k = 1; k < K; ++k) {
        const long long want = nnz * k / K;
        int lo = r[k - 1], hi = m;   // first row with ptr[row] >= want
        while (lo < hi) {
            const int mid = lo + (hi - lo) / 2;
            if (c.ptr[mid] >= want) hi = mid; else lo = mid + 1;
        }
        r[k] = lo;
    }
    const size_t pad = 256;
    double *d_val = static_cast<double *>(device_scratch(1, sizeof(double) * (size_t)nnz + K * pad));
    int *d_idx = static_cast<int *>(device_scratch(2, sizeof(int) * (size_t)nnz + K * pad));
    int *d_ptr = static_cast<int *>(device_scratch(3, sizeof(int) * (size_t)(m + 1)));
    double *d_x = static_cast<double *>(device_scratch(4, sizeof(double) * (size_t)n));
    double *d_y = static_cast<double *>(device_scratch(5, sizeof(double) * (size_t)m));
    int *d_rp = static_cast<int *>(device_scratch(8, sizeof(int) * (size_t)(m + 1 + K) + K * pad));
    const int sigma = (c.kernel == 3) ? csr5_sigma_for(m, nnz) : default_sigma_for(m, nnz);
    void *w = device_scratch(0, tile_workspace_bytes(nnz, sigma));
    if (!d_val || !d_idx || !d_ptr || !d_x || !d_y || !d_rp || !w) {
        set_error(SBLAS_ERR_ALLOC, "%s: device allocation failed", c.name);
        return failed();
    }
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    cudaEvent_t e0 = ctx->ev[0], e1 = ctx->ev[1], e2 = ctx->ev[2], e3 = ctx->ev[3];
    // ---- inputs every chunk needs: row pointer, x (and y when it is read)
    DROPIN_CUDA(cudaEventRecord(e0, cs));
    DROPIN_CUDA(cudaMemcpyAsync(d_ptr, c.ptr, sizeof(int) * (size_t)(m + 1), cudaMemcpyHostToDevice, cs));
    DROPIN_CUDA(cudaMemcpyAsync(d_x, c.x, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, cs));
    if (need_y_in)
        DROPIN_CUDA(cudaMemcpyAsync(d_y, c.y, sizeof(double) * (size_t)m, cudaMemcpyHostToDevice, cs));
    DROPIN_CUDA(cudaEventRecord(ctx->chunk_ev[0], cs));
    // ---- the chunks' values and columns
    size_t vo[kPipeChunks], io[kPipeChunks], ro[kPipeChunks];
    size_t voff = 0, ioff = 0, roff = 0;
    for (int k = 0; k < K; ++k) {
        const long long lo = c.ptr[r[k]], hi = c.ptr[r[k + 1]];
        vo[k] = voff;
        io[k] = ioff;
        ro[k] = roff;
        if (hi > lo) {
            DROPIN_CUDA(cudaMemcpyAsync(reinterpret_cast<unsigned char *>(d_val) + voff, c.val + lo,
                                        sizeof(double) * (size_t)(hi - lo), cudaMemcpyHostToDevice, cs));
            DROPIN_CUDA(cudaMemcpyAsync(reinterpret_cast<unsigned char *>(d_idx) + ioff, c.idx + lo,
                                        sizeof(int) * (size_t)(hi - lo), cudaMemcpyHostToDevice, cs));
        }
        DROPIN_CUDA(cudaEventRecord(ctx->chunk_ev[1 + k], cs));
        voff += up(sizeof(double) * (size_t)(hi - lo));
        ioff += up(sizeof(int) * (size_t)(hi - lo));
        roff += up(sizeof(int) * (size_t)(r[k + 1] - r[k] + 1));
    }
    DROPIN_CUDA(cudaEventRecord(e1, cs));
    // ---- per chunk: rebase its row pointer, SpMV, send its rows of y back
    DROPIN_CUDA(cudaStreamWaitEvent(ks, ctx->chunk_ev[0], 0));
    DROPIN_CUDA(cudaEventRecord(e2, ks));
    const double beta_eff = c.additive ? c.beta + 1.0 : c.beta;
    bool status_cleared = false;
    for (int k = 0; k < K; ++k) {
        const int rows = r[k + 1] - r[k];
        if (rows == 0) continue;
        const long long lo = c.ptr[r[k]], cnnz = c.ptr[r[k + 1]] - lo;
        int *rp = reinterpret_cast<int *>(reinterpret_cast<unsigned char *>(d_rp) + ro[k]);
        rebase_rowptr_kernel<<<(rows + 1 + 255) / 256 < 1024 ? (rows + 1 + 255) / 256 : 1024, 256, 0, ks>>>(
            rows + 1, d_ptr + r[k], (int)lo, rp);
        DROPIN_CUDA(cudaGetLastError());
        DROPIN_CUDA(cudaStreamWaitEvent(ks, ctx->chunk_ev[1 + k], 0));
        const double *val = reinterpret_cast<const double *>(reinterpret_cast<unsigned char *>(d_val) + vo[k]);
        const int *col = reinterpret_cast<const int *>(reinterpret_cast<unsigned char *>(d_idx) + io[k]);
        // the chunks share one workspace: its status word is cleared once,
        // by the first launch, so a chunk that gave up a wait stays visible
        const int rc = (cnnz == 0)
                           ? launch_scale_y(rows, beta_eff, d_y + r[k], ks)
                           : launch_tile_spmv(rows, n, cnnz, c.alpha, val, SBLAS_VAL_F64, rp, col, d_x,
                                              beta_eff, d_y + r[k], sigma, w, ks, false,
                                              !status_cleared);
        if (cnnz > 0) status_cleared = true;
        if (rc != SBLAS_OK) return failed();
        DROPIN_CUDA(cudaMemcpyAsync(c.y + r[k], d_y + r[k], sizeof(double) * (size_t)rows,
                                    cudaMemcpyDeviceToHost, ks));
    }
    DROPIN_CUDA(cudaEventRecord(e3, ks));
    const double tm = wall();
    DROPIN_CUDA(cudaEventSynchronize(e3));
    if (!launches_completed(c, w)) return failed();
    spmv_ret ret = zero_ret();
    float t_comm = 0.f, t_comp = 0.f;
    DROPIN_CUDA(cudaEventElapsedTime(&t_comm, e0, e1));
    DROPIN_CUDA(cudaEventElapsedTime(&t_comp, e2, e3));
    ret.comm_time = t_comm * 1e-3;   // host-to-device copies (overlapping the kernels)
    ret.comp_time = t_comp * 1e-3;   // kernels and the copies of y back, from the first chunk on
    ret.merg_time = wall() - tm;
    return ret;
}

// The engine behind every host entry point.
spmv_ret run_host(Call c)
{
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    DeviceContext *ctx = device_context();
    if (!ctx) {
        set_error(SBLAS_ERR_CUDA, "%s: no usable CUDA device", c.name);
        return failed();
    }
    spmv_ret ret = zero_ret();
    if (c.m == 0) return ret;
    if (c.fmt == Fmt::CSR && c.kernel != 1 && c.nnz >= kPipeMinNnz && c.n > 0 && c.row_lo == 0 &&
        c.row_hi == c.m)
        return run_host_pipelined(c, ctx);
    cudaStream_t st = ctx->stream;
    const int m = c.m, n = c.n;
    const long long nnz = c.nnz;
    const int nptr = (c.fmt == Fmt::CSC) ? n + 1 : (c.fmt == Fmt::CSR ? m + 1 : 0);
    const bool need_y_in = (c.beta != 0.0) || c.additive;

    // device buffers (grow-only, reused across calls)
    double *d_val = static_cast<double *>(device_scratch(1, sizeof(double) * (size_t)nnz));
    int *d_idx = static_cast<int *>(device_scratch(2, sizeof(int) * (size_t)nnz));
    int *d_ptr = static_cast<int *>(device_scratch(3, sizeof(int) * (size_t)(nptr > 0 ? nptr : (nnz > 0 ? nnz : 1))));
    double *d_x = static_cast<double *>(device_scratch(4, sizeof(double) * (size_t)(n > 0 ? n : 1)));
    double *d_y = static_cast<double *>(device_scratch(5, sizeof(double) * (size_t)m));
    if (!d_val || !d_idx || !d_ptr || !d_x || !d_y) {
        set_error(SBLAS_ERR_ALLOC, "%s: device allocation failed", c.name);
        return failed();
    }
    cudaEvent_t e0 = ctx->ev[0], e1 = ctx->ev[1], e2 = ctx->ev[2], e3 = ctx->ev[3];
    // ---- host -> device
    DROPIN_CUDA(cudaEventRecord(e0, st));
    if (nnz > 0) {
        DROPIN_CUDA(cudaMemcpyAsync(d_val, c.val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
        DROPIN_CUDA(cudaMemcpyAsync(d_idx, c.idx, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
        DROPIN_CUDA(cudaMemcpyAsync(d_x, c.x, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    }
    if (c.fmt != Fmt::COO)
        DROPIN_CUDA(cudaMemcpyAsync(d_ptr, c.ptr, sizeof(int) * nptr, cudaMemcpyHostToDevice, st));
    else if (nnz > 0)
        DROPIN_CUDA(cudaMemcpyAsync(d_ptr, c.ptr, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
    if (need_y_in)
        DROPIN_CUDA(cudaMemcpyAsync(d_y, c.y, sizeof(double) * m, cudaMemcpyHostToDevice, st));
    DROPIN_CUDA(cudaEventRecord(e1, st));

    // ---- format work: CSC -> CSR, COO rows -> row pointer
    const int *rowptr = d_ptr;
    const int *col = d_idx;
    const double *val = d_val;
    const bool csc_direct = (c.fmt == Fmt::CSC);   // summed by row blocks, no CSR copy
    if (c.fmt == Fmt::COO) {
        int *o_ptr = static_cast<int *>(device_scratch(7, sizeof(int) * (size_t)(m + 1)));
        if (!o_ptr || launch_coo_rows_to_rowptr(m, nnz, d_ptr, o_ptr, st) != SBLAS_OK)
            return failed();
        rowptr = o_ptr;
    }
    DROPIN_CUDA(cudaEventRecord(e2, st));

    // ---- the SpMV on rows [row_lo, row_hi)
    const int rows = c.row_hi - c.row_lo;
    const double beta_eff = c.additive ? c.beta + 1.0 : c.beta;
    void *tile_work = nullptr;   // workspace of the tile launch, if one ran
    if (csc_direct && rows > 0) {
        // the CSC product: the row-ordered structure by a stable bucket sort
        // (inspector), then the values in row order and the tile kernel
        const size_t wb = cscmv_workspace_bytes(m, n, nnz);
        void *w = device_scratch(6, wb);
        if (!w) {
            set_error(SBLAS_ERR_ALLOC, "%s: workspace allocation failed", c.name);
            return failed();
        }
        if (launch_csc_analyse(m, n, nnz, d_ptr, d_idx, w, wb, false, st) != SBLAS_OK)
            return failed();
        DROPIN_CUDA(cudaEventRecord(e2, st));   // the inspector counts as format work
        if (launch_cscmv_analysed(m, n, nnz, c.alpha, d_val, d_x, beta_eff, d_y, w, wb, false,
                                  st) != SBLAS_OK)
            return failed();
        if (nnz > 0 && n > 0) tile_work = csc_tile_workspace(w, m, n, nnz);
    } else if (rows > 0) {
        // a row sub-range keeps absolute offsets into col/val
        const int *rp = rowptr + c.row_lo;
        double *yp = d_y + c.row_lo;
        int rc;
        if (nnz == 0) {
            rc = launch_scale_y(rows, beta_eff, yp, st);
        } else if (c.kernel == 1) {
            rc = launch_rowsplit_spmv(rows, n, nnz, c.alpha, val, rp, col, d_x, beta_eff, yp, st);
        } else {
            const int tile_sigma =
                (c.kernel == 3) ? csr5_sigma_for(m, nnz) : default_sigma_for(m, nnz);
            tile_work = device_scratch(0, tile_workspace_bytes(nnz, tile_sigma));
            if (!tile_work) {
                set_error(SBLAS_ERR_ALLOC, "%s: workspace allocation failed", c.name);
                return failed();
            }
            rc = launch_tile_spmv(rows, n, nnz, c.alpha, val, SBLAS_VAL_F64, rp, col, d_x,
                                  beta_eff, yp, tile_sigma, tile_work, st);
        }
        if (rc != SBLAS_OK) return failed();
    }
    DROPIN_CUDA(cudaEventRecord(e3, st));
    DROPIN_CUDA(cudaEventSynchronize(e3));
    if (tile_work && !launches_completed(c, tile_work)) return failed();
    float t_comm = 0.f, t_part = 0.f, t_comp = 0.f;
    DROPIN_CUDA(cudaEventElapsedTime(&t_comm, e0, e1));
    DROPIN_CUDA(cudaEventElapsedTime(&t_part, e1, e2));
    DROPIN_CUDA(cudaEventElapsedTime(&t_comp, e2, e3));

    // ---- device -> host: only the rows this call writes
    const double tm = wall();
    if (rows > 0)
        DROPIN_CUDA(cudaMemcpyAsync(c.y + c.row_lo, d_y + c.row_lo, sizeof(double) * rows,
                                    cudaMemcpyDeviceToHost, st));
    DROPIN_CUDA(cudaStreamSynchronize(st));
    ret.merg_time = wall() - tm;
    ret.comm_time = t_comm * 1e-3;
    ret.part_time = t_part * 1e-3;
    ret.comp_time = t_comp * 1e-3;
    return ret;
}

// Rows an nnz-split entry point writes in reference-compatibility mode: the
// rows holding the first and the last nonzero (src/dspmv_mgpu_v1.cu:132-157
// with one part).
void nnz_split_rows(const int *rowptr, int m, long long nnz, int *lo, int *hi)
{
    if (nnz <= 0) {
        *lo = 0;
        *hi = m;
        return;
    }
    *lo = row_of_index(m, rowptr, 0);
    *hi = row_of_index(m, rowptr, (int)(nnz - 1)) + 1;
}

spmv_ret csr_entry(const char *name, int m, int n, long long nnz, double *alpha, double *val,
                   int *rowptr, int *col, double *x, double *beta, double *y, int ngpu,
                   int kernel, bool nnz_split, bool additive_in_compat)
{
    clear_error();
    if (!check_common(name, m, n, nnz, alpha, beta, val, rowptr, col, x, y, ngpu) ||
        !check_kernel(name, kernel))
        return failed();
    const bool compat = sblas_get_compat_mode() != 0;
    Call c{name, Fmt::CSR, m, n, nnz, *alpha, *beta, val, rowptr, col, x, y, kernel, 0, m, false};
    if (compat) {
        if (nnz_split) nnz_split_rows(rowptr, m, nnz, &c.row_lo, &c.row_hi);
        if (kernel == 3) {  // CSR5 path computes y = A*x (csr5_spmv_cuda.h:22)
            c.alpha = 1.0;
            c.beta = 0.0;
        }
        c.additive = additive_in_compat;
    }
    return run_host(c);
}

}  // namespace
}  // namespace sblas

using namespace sblas;

extern "C" {

spmv_ret spMV_mgpu_baseline(int m, int n, int nnz, double *alpha, double *csrVal, int *csrRowPtr,
                            int *csrColIndex, double *x, double *beta, double *y, int ngpu)
{
    return csr_entry("spMV_mgpu_baseline", m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x,
                     beta, y, ngpu, SBLAS_KERNEL_MERGEPATH, false, false);
}

spmv_ret spMV_mgpu_v1(int m, int n, int nnz, double *alpha, double *csrVal, int *csrRowPtr,
                      int *csrColIndex, double *x, double *beta, double *y, int ngpu, int kernel)
{
    return csr_entry("spMV_mgpu_v1", m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta,
                     y, ngpu, kernel, true, false);
}

spmv_ret spMV_mgpu_v1_numa(int m, int n, int nnz, double *alpha, double *csrVal, int *csrRowPtr,
                           int *csrColIndex, double *x, double *beta, double *y, int ngpu,
                           int kernel, int *numa_mapping, int part_opt, int merg_opt)
{
    clear_error();
    if ((part_opt != 0 && part_opt != 1) || (merg_opt != 0 && merg_opt != 1)) {
        set_error(SBLAS_ERR_ARG, "spMV_mgpu_v1_numa: part_opt and merg_opt must be 0 or 1");
        return failed();
    }
    if (numa_mapping && numa_mapping[0] < 0) {
        set_error(SBLAS_ERR_ARG, "spMV_mgpu_v1_numa: negative NUMA node");
        return failed();
    }
    // the reference always runs csrmv here (src/dspmv_mgpu_v1_numa.cu:696)
    (void)kernel;
    return csr_entry("spMV_mgpu_v1_numa", m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x,
                     beta, y, ngpu, SBLAS_KERNEL_MERGEPATH, true, merg_opt == 0);
}

spmv_ret spMV_mgpu_v2(int m, int n, int nnz, double *alpha, double *csrVal, int *csrRowPtr,
                      int *csrColIndex, double *x, double *beta, double *y, int ngpu, int kernel,
                      int nb, int copy_of_workspace)
{
    clear_error();
    if (nb <= 0 || copy_of_workspace <= 0) {
        set_error(SBLAS_ERR_ARG, "spMV_mgpu_v2: nb and copy_of_workspace must be positive");
        return failed();
    }
    // The reference's task pool of nb-nonzero chunks on q streams
    // (src/dspmv_mgpu_v2.cu:103-307) is one persistent tile kernel here.
    return csr_entry("spMV_mgpu_v2", m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta,
                     y, ngpu, kernel, true, false);
}

spmv_ret spMV_mgpu_baseline_csc(int m, int n, int nnz, double *alpha, double *cscVal,
                                int *cscColPtr, int *cscRowIdx, double *x, double *beta,
                                double *y, int ngpu)
{
    clear_error();
    if (!check_common("spMV_mgpu_baseline_csc", m, n, nnz, alpha, beta, cscVal, cscColPtr,
                      cscRowIdx, x, y, ngpu))
        return failed();
    Call c{"spMV_mgpu_baseline_csc", Fmt::CSC, m, n, nnz, *alpha, *beta, cscVal, cscColPtr,
           cscRowIdx, x, y, SBLAS_KERNEL_MERGEPATH, 0, m, false};
    // the reference adds the device result into y (baseline_csc.cu:171-175)
    c.additive = sblas_get_compat_mode() != 0;
    return run_host(c);
}

spmv_ret spMV_mgpu_v1_numa_csc(int m, int n, long long nnz, double *alpha, double *cscVal,
                               int *cscColPtr, int *cscRowIndex, double *x, double *beta,
                               double *y, int ngpu, int kernel, int *numa_mapping, int part_opt,
                               int merg_opt)
{
    clear_error();
    (void)kernel;
    (void)numa_mapping;
    if ((part_opt != 0 && part_opt != 1) || (merg_opt != 0 && merg_opt != 1)) {
        set_error(SBLAS_ERR_ARG, "spMV_mgpu_v1_numa_csc: part_opt and merg_opt must be 0 or 1");
        return failed();
    }
    if (!check_common("spMV_mgpu_v1_numa_csc", m, n, nnz, alpha, beta, cscVal, cscColPtr,
                      cscRowIndex, x, y, ngpu))
        return failed();
    Call c{"spMV_mgpu_v1_numa_csc", Fmt::CSC, m, n, nnz, *alpha, *beta, cscVal, cscColPtr,
           cscRowIndex, x, y, SBLAS_KERNEL_MERGEPATH, 0, m, false};
    // both merge options add into y (src/dspmv_mgpu_v1_numa_csc.cu, merge section)
    c.additive = sblas_get_compat_mode() != 0;
    return run_host(c);
}

spmv_ret spMV_mgpu_baseline_coo(int m, int n, int nnz, double *alpha, double *cooVal,
                                int *cooRowIdx, int *cooColIdx, double *x, double *beta,
                                double *y, int ngpu)
{
    clear_error();
    if (!check_common("spMV_mgpu_baseline_coo", m, n, nnz, alpha, beta, cooVal, cooRowIdx,
                      cooColIdx, x, y, ngpu))
        return failed();
    Call c{"spMV_mgpu_baseline_coo", Fmt::COO, m, n, nnz, *alpha, *beta, cooVal, cooRowIdx,
           cooColIdx, x, y, SBLAS_KERNEL_MERGEPATH, 0, m, false};
    return run_host(c);
}

spmv_ret spMV_mgpu_v1_numa_coo(int m, int n, int nnz, double *alpha, double *cooVal,
                               int *cooRowIdx, int *cooColIdx, double *x, double *beta,
                               double *y, int ngpu, int kernel, int *numa_mapping, int part_opt,
                               int merg_opt)
{
    clear_error();
    (void)kernel;
    (void)numa_mapping;
    if ((part_opt != 0 && part_opt != 1) || (merg_opt != 0 && merg_opt != 1)) {
        set_error(SBLAS_ERR_ARG, "spMV_mgpu_v1_numa_coo: part_opt and merg_opt must be 0 or 1");
        return failed();
    }
    if (!check_common("spMV_mgpu_v1_numa_coo", m, n, nnz, alpha, beta, cooVal, cooRowIdx,
                      cooColIdx, x, y, ngpu))
        return failed();
    Call c{"spMV_mgpu_v1_numa_coo", Fmt::COO, m, n, nnz, *alpha, *beta, cooVal, cooRowIdx,
           cooColIdx, x, y, SBLAS_KERNEL_MERGEPATH, 0, m, false};
    if (sblas_get_compat_mode() != 0 && nnz > 0) {
        // rows of the first and last nonzero (dspmv_mgpu_v1_numa_coo.cu:64-65)
        c.row_lo = cooRowIdx[0];
        c.row_hi = cooRowIdx[nnz - 1] + 1;
        c.additive = (merg_opt == 0);
    }
    return run_host(c);
}

// SpMSpV: the nonzeros whose x entry is zero are dropped on the host before
// the SpMV, as src/dspmv_mgpu_v1.cu:19-74 does.
// spMspV's x-zero filter (src/dspmv_mgpu_v1.cu:29-40) on all host threads:
// the rows are cut into blocks of about equal nonzeros, every block counts
// its kept nonzeros, an exclusive prefix of the counts gives every block its
// output offset, and every block then writes its rows.  The output equals
// the reference's serial loop.
static void host_filter_x(int m, const int *rowptr, const int *col, const double *val,
                          const double *x, std::vector<int> &rp, std::vector<int> &rc,
                          std::vector<double> &rv)
{
    if (m <= 0 || rowptr == nullptr) {   // no rows: an empty matrix (rowptr may be null)
        rp.assign(1, 0);
        rc.clear();
        rv.clear();
        return;
    }
    const long long nnz = (long long)rowptr[m] - rowptr[0];
    int T = (int)std::thread::hardware_concurrency();
    T = std::max(1, std::min(T, 64));
    if (nnz < (1LL << 20)) T = 1;
    std::vector<int> rb(T + 1);
    rb[0] = 0;
    rb[T] = m;
    for (int t = 1; t < T; ++t) {
        const long long target = rowptr[0] + nnz * t / T;
        const int r = (int)(std::upper_bound(rowptr, rowptr + m + 1, (int)target) - rowptr) - 1;
        rb[t] = std::min(m, std::max(rb[t - 1], r));
    }
    std::vector<long long> first(T + 1, 0);
    auto run = [&](auto &&body) {
        if (T == 1) {
            body(0);
            return;
        }
        std::vector<std::thread> th;
        th.reserve(T);
        for (int t = 0; t < T; ++t) th.emplace_back(body, t);
        for (auto &h : th) h.join();
    };
    run([&](int t) {
        long long c = 0;
        for (int j = rowptr[rb[t]]; j < rowptr[rb[t + 1]]; ++j) c += (x[col[j]] != 0.0);
        first[t + 1] = c;
    });
    for (int t = 0; t < T; ++t) first[t + 1] += first[t];
    rp.assign((size_t)m + 1, 0);
    rc.resize((size_t)first[T]);
    rv.resize((size_t)first[T]);
    run([&](int t) {
        long long k = first[t];
        for (int i = rb[t]; i < rb[t + 1]; ++i) {
            for (int j = rowptr[i]; j < rowptr[i + 1]; ++j)
                if (x[col[j]] != 0.0) {
                    rc[(size_t)k] = col[j];
                    rv[(size_t)k] = val[j];
                    ++k;
                }
            rp[(size_t)i + 1] = (int)k;
        }
    });
}

static spmv_ret spmspv(const char *name, int m, int n, int nnz, double *alpha, double *val,
                       int *rowptr, int *col, double *x, double *beta, double *y, int ngpu,
                       int kernel, int v2, int nb, int q)
{
    clear_error();
    if (!check_common(name, m, n, nnz, alpha, beta, val, rowptr, col, x, y, ngpu) ||
        !check_kernel(name, kernel))
        return failed();
    const double t0 = wall();
    std::vector<double> rv;
    std::vector<int> rc, rp;
    host_filter_x(m, rowptr, col, val, x, rp, rc, rv);
    const double filt = wall() - t0;
    spmv_ret r = v2 ? spMV_mgpu_v2(m, n, (int)rv.size(), alpha, rv.data(), rp.data(), rc.data(),
                                   x, beta, y, ngpu, kernel, nb, q)
                    : spMV_mgpu_v1(m, n, (int)rv.size(), alpha, rv.data(), rp.data(), rc.data(),
                                   x, beta, y, ngpu, kernel);
    if (r.comp_time >= 0) r.part_time += filt;
    return r;
}

spmv_ret spMspV_mgpu_v1(int m, int n, int nnz, double *alpha, double *csrVal, int *csrRowPtr,
                        int *csrColIndex, double *x, double *beta, double *y, int ngpu,
                        int kernel)
{
    return spmspv("spMspV_mgpu_v1", m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta, y,
                  ngpu, kernel, 0, 1, 1);
}

spmv_ret spMspV_mgpu_v2(int m, int n, int nnz, double *alpha, double *csrVal, int *csrRowPtr,
                        int *csrColIndex, double *x, double *beta, double *y, int ngpu,
                        int kernel, int nb, int copy_of_workspace)
{
    return spmspv("spMspV_mgpu_v2", m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta, y,
                  ngpu, kernel, 1, nb, copy_of_workspace);
}

int csr5_kernel(int m, int n, int nnz, double *alpha, double *csrVal, int *csrRowPtr,
                int *csrColIndex, double *x, double *beta, double *y,
                sblas_cuda_stream_t stream)
{
    clear_error();
    if (!alpha || !beta) {
        set_error(SBLAS_ERR_ARG, "csr5_kernel: alpha and beta must be non-null");
        return SBLAS_ERR_ARG;
    }
    const bool compat = sblas_get_compat_mode() != 0;
    const double a = compat ? 1.0 : *alpha, b = compat ? 0.0 : *beta;
    return sblas_dcsrmv(SBLAS_KERNEL_CSR5, m, n, nnz, a, csrVal, SBLAS_VAL_F64, csrRowPtr,
                        csrColIndex, x, b, y, csr5_sigma_for(m, nnz), nullptr, 0,
                        reinterpret_cast<void *>(stream));
}

// ---- helpers -------------------------------------------------------------

int get_row_from_index(int n, int *a, int idx) { return row_of_index(n, a, idx); }

double get_time(void) { return wall(); }

double get_gpu_availble_mem(int ngpu)
{
    double best = -1.0;
    int cur = 0;
    cudaGetDevice(&cur);
    for (int d = 0; d < ngpu; ++d) {
        size_t fr = 0, tot = 0;
        if (cudaSetDevice(d) != cudaSuccess || cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        const double gb = (double)fr / 1e9;
        if (best < 0 || gb < best) best = gb;
    }
    cudaSetDevice(cur);
    return best;
}

int findFirstInSorted(int *a, int n, int key)
{
    // src/spmv_helper.cu:646-665
    int l = 0, r = n;
    while (l < r - 1) {
        const int mid = l + (r - l) / 2;
        if (key <= a[mid]) r = mid;
        else l = mid;
    }
    if (key == a[l]) return l;
    if (key == a[r]) return r;
    return l;
}

int findLastInSorted(int *a, int n, int key)
{
    // src/spmv_helper.cu:668-685
    int l = 0, r = n;
    while (l < r - 1) {
        const int mid = l + (r - l) / 2;
        if (key < a[mid]) r = mid;
        else l = mid;
    }
    if (key == a[l]) return l;
    if (key == a[r]) return r;
    return l;
}

}  // extern "C"

namespace sblas {
namespace {
// Stable device sort of a host COO matrix by row (by_row) or by column; the
// sorted triplets go to oval/orow/ocol (may alias the inputs) and, when
// optr is non-null, the compressed pointer of the sort key (nkeys + 1).
// Same result as the reference's cuSPARSE coosort + coo2csr
// (src/spmv_helper.cu:277-387, :493-642): a stable sort by the key index
// carrying the other index and the value (this library's bucket passes).
int host_coo_sort(int m, int n, int nnz, const double *val, const int *row, const int *col,
                  bool by_row, double *oval, int *orow, int *ocol, int *optr)
{
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (m < 0 || n < 0 || nnz < 0 || (nnz > 0 && (!val || !row || !col))) {
        set_error(SBLAS_ERR_ARG, "COO sort: bad arguments");
        return SBLAS_ERR_ARG;
    }
    DeviceContext *ctx = device_context();
    if (!ctx) {
        set_error(SBLAS_ERR_CUDA, "no usable CUDA device");
        return SBLAS_ERR_CUDA;
    }
    cudaStream_t st = ctx->stream;
    const int nkeys = by_row ? m : n;
    const size_t nb = (size_t)(nnz > 0 ? nnz : 1);
    double *d_val = static_cast<double *>(device_scratch(1, sizeof(double) * nb));
    int *d_row = static_cast<int *>(device_scratch(2, sizeof(int) * nb));
    int *d_col = static_cast<int *>(device_scratch(3, sizeof(int) * nb));
    int *d_keys = static_cast<int *>(device_scratch(8, sizeof(int) * nb));
    const size_t wb = coo_sort_workspace_bytes(nkeys, nnz);
    void *d_work = device_scratch(10, wb);
    int *d_other = static_cast<int *>(device_scratch(11, sizeof(int) * nb));
    double *d_oval = static_cast<double *>(device_scratch(12, sizeof(double) * nb));
    int *d_ptr = static_cast<int *>(device_scratch(13, sizeof(int) * (size_t)(nkeys + 1)));
    if (!d_val || !d_row || !d_col || !d_keys || !d_work || !d_other || !d_oval || !d_ptr) {
        set_error(SBLAS_ERR_ALLOC, "COO sort: device allocation failed");
        return SBLAS_ERR_ALLOC;
    }
    if (nnz > 0) {
        SBLAS_CUDA_TRY(cudaMemcpyAsync(d_val, val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
        SBLAS_CUDA_TRY(cudaMemcpyAsync(d_row, row, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
        SBLAS_CUDA_TRY(cudaMemcpyAsync(d_col, col, sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
    }
    const int *keys = by_row ? d_row : d_col;
    const int *other = by_row ? d_col : d_row;
    int rc = launch_coo_sort(nkeys, nnz, keys, other, d_val, d_keys, d_other, d_oval, d_work, wb,
                             st);
    if (rc == SBLAS_OK && optr) rc = launch_coo_rows_to_rowptr(nkeys, nnz, d_keys, d_ptr, st);
    if (rc != SBLAS_OK) return rc;
    if (nnz > 0) {
        SBLAS_CUDA_TRY(cudaMemcpyAsync(oval, d_oval, sizeof(double) * nnz, cudaMemcpyDeviceToHost, st));
        int *okey = by_row ? orow : ocol;
        int *oother = by_row ? ocol : orow;
        if (okey)
            SBLAS_CUDA_TRY(cudaMemcpyAsync(okey, d_keys, sizeof(int) * nnz, cudaMemcpyDeviceToHost, st));
        SBLAS_CUDA_TRY(cudaMemcpyAsync(oother, d_other, sizeof(int) * nnz, cudaMemcpyDeviceToHost, st));
    }
    if (optr)
        SBLAS_CUDA_TRY(cudaMemcpyAsync(optr, d_ptr, sizeof(int) * (size_t)(nkeys + 1),
                                       cudaMemcpyDeviceToHost, st));
    SBLAS_CUDA_TRY(cudaStreamSynchronize(st));
    return SBLAS_OK;
}
}  // namespace
}  // namespace sblas

extern "C" {

void sortCOORow(int m, int n, int nnz, double *cooVal, int *cooRowIdx, int *cooColIdx)
{
    clear_error();
    host_coo_sort(m, n, nnz, cooVal, cooRowIdx, cooColIdx, true, cooVal, cooRowIdx, cooColIdx,
                  nullptr);
}

void sortCOOCol(int m, int n, int nnz, double *cooVal, int *cooRowIdx, int *cooColIdx)
{
    clear_error();
    host_coo_sort(m, n, nnz, cooVal, cooRowIdx, cooColIdx, false, cooVal, cooRowIdx, cooColIdx,
                  nullptr);
}

void coo2csr(int m, int n, int nnz, double *cooVal, int *cooRowIdx, int *cooColIdx,
             double *csrVal, int *csrRowPtr, int *csrColIdx)
{
    clear_error();
    host_coo_sort(m, n, nnz, cooVal, cooRowIdx, cooColIdx, true, csrVal, nullptr, csrColIdx,
                  csrRowPtr);
}

void coo2csc(int m, int n, int nnz, double *cooVal, int *cooRowIdx, int *cooColIdx,
             double *cscVal, int *cscColPtr, int *cscRowIdx)
{
    clear_error();
    host_coo_sort(m, n, nnz, cooVal, cooRowIdx, cooColIdx, false, cscVal, cscRowIdx, nullptr,
                  cscColPtr);
}

void coo2csrGPU(void *handle, sblas_cuda_stream_t stream, int m, int n, int nnz, double *cooVal,
                int *cooRowIdx, int *cooColIdx, double *csrVal, int *csrRowPtr, int *csrColIdx)
{
    // src/spmv_helper.cu:478-490: row pointer from row-sorted COO, then copies
    (void)handle;
    (void)n;
    clear_error();
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (launch_coo_rows_to_rowptr(m, nnz, cooRowIdx, csrRowPtr, st) != SBLAS_OK) return;
    if (nnz > 0) {
        cudaMemcpyAsync(csrVal, cooVal, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(csrColIdx, cooColIdx, sizeof(int) * nnz, cudaMemcpyDeviceToDevice, st);
    }
}

void report_mem_usage(int d)
{
    size_t fr = 0, tot = 0;
    int cur = 0;
    cudaGetDevice(&cur);
    if (cudaSetDevice(d) == cudaSuccess && cudaMemGetInfo(&fr, &tot) == cudaSuccess)
        printf("GPU %d memory usage: used = %f, free = %f MB, total = %f MB\n", d,
               (double)(tot - fr) / 1048576.0, (double)fr / 1048576.0, (double)tot / 1048576.0);
    cudaSetDevice(cur);
}

void report_all_mem_usage(void)
{
    int cnt = 0;
    if (cudaGetDeviceCount(&cnt) != cudaSuccess) return;
    for (int d = 0; d < cnt; ++d) report_mem_usage(d);
}

void print_vec_double(double *a, int n, const char *s)
{
    printf("%s: ", s ? s : "");
    for (int i = 0; i < n; ++i) printf("%g ", a[i]);
    printf("\n");
}

void print_vec_int(int *a, int n, const char *s)
{
    printf("%s: ", s ? s : "");
    for (int i = 0; i < n; ++i) printf("%d ", a[i]);
    printf("\n");
}

void print_vec_gpu_double(double *a, int n, const char *s)
{
    std::vector<double> h((size_t)(n > 0 ? n : 0));
    if (n > 0) cudaMemcpy(h.data(), a, sizeof(double) * n, cudaMemcpyDeviceToHost);
    print_vec_double(h.data(), n, s);
}

void print_vec_gpu_int(int *a, int n, const char *s)
{
    std::vector<int> h((size_t)(n > 0 ? n : 0));
    if (n > 0) cudaMemcpy(h.data(), a, sizeof(int) * n, cudaMemcpyDeviceToHost);
    print_vec_int(h.data(), n, s);
}

}  // extern "C"
