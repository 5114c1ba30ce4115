// Internal declarations shared by the CUDA translation units of
// libsblas_gb300.so.  Nothing here is part of the public C ABI
// (include/sblas_gb300.h and include/spmv_kernel.h are).
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "../../include/sblas_gb300.h"

namespace sblas {

// ---- error state: thread-local status readable through sblas_last_error ----
void set_error(int code, const char *fmt, ...);
void clear_error();
int last_status();

#define SBLAS_CUDA_TRY(expr)                                                          \
    do {                                                                              \
        cudaError_t sblas_e_ = (expr);                                                \
        if (sblas_e_ != cudaSuccess) {                                                \
            ::sblas::set_error(SBLAS_ERR_CUDA, "%s failed: %s (%s:%d)", #expr,      \
                               cudaGetErrorString(sblas_e_), __FILE__, __LINE__);    \
            return SBLAS_ERR_CUDA;                                                    \
        }                                                                             \
    } while (0)

// ---- nnz-tile engine (the load-balanced CSR kernel) ----------------------
// A tile is TILE_THREADS * sigma consecutive nonzeros.  Workspace per call:
//   status[1]             device error flag (bounded waits), first 256 bytes
//   row_part[ntiles + 1]  first owned row of every tile (int32)
//   carry[ntiles]         FP64 partial of the row that continues past the tile
struct TileShape {
    int threads;   // threads per CTA
    int sigma;     // nonzeros per thread
    long long tile() const { return (long long)threads * sigma; }
};

// Shapes compiled into the library (sigma odd: conflict-free shared reads).
int tile_shape_count();
TileShape tile_shape_at(int i);
int tile_shape_index(int sigma);   // -1 if not compiled

size_t tile_workspace_bytes(long long nnz, int sigma);

// Value storage of the matrix:  0 = FP64, 1 = FP32 (widened to FP64, products
// and sums in FP64), 2 = pattern (no value array; every stored entry is 1).
enum ValueKind { VAL_F64 = 0, VAL_F32 = 1, VAL_PATTERN = 2 };

// Launches partition + tile kernel + carry fix-up on `stream`.
// `work` must hold tile_workspace_bytes(nnz, sigma) bytes, 256-byte aligned.
// analysed = true: the partition of `work` was computed by
// launch_tile_analyse for this row pointer and sigma (skipped here).
// reset_status = false keeps the workspace's status word as it is (a call
// made of several launches on one workspace clears it once, at its start).
int launch_tile_spmv(int m, int n, long long nnz, double alpha, const void *val,
                     int val_kind, const int *rowptr, const int *col, const double *x,
                     double beta, double *y, int sigma, void *work, cudaStream_t stream,
                     bool analysed = false, bool reset_status = true);
// Status word of a tile workspace (0 = every wait completed), read with a
// synchronous copy: the caller has synchronised the launches' stream.
int tile_workspace_status(void *work, int *out);
// The sticky per-device word (any tile launch that gave up a wait), read
// after `stream` completes; clear = reset it to 0.
int tile_sticky_status(cudaStream_t stream, bool clear, int *out);
// Bounded-wait limit of the tile kernels (0 = the default, 2 s) and the
// test hook that keeps the producer warp from staging (waits then run out).
// The tile kernel over several matrices in one launch (the batched form
// with one right-hand side): global tiles [0, ntiles), matrix i owning
// tiles [tile0s[i], tile0s[i+1]) and partition entries part[part_off_i ..
// part_off_i + its tiles]; every matrix has at least one tile.  mats: device
// array of descriptors written by fill_multi_mat.
struct MultiTileLaunch {
    const void *mats;
    const int *tile0s;   // [nmat + 1]
    int nmat;
    int ntiles;
    const int *part;
    double *carry;       // [ntiles]
    int *status;
};
int multi_tile_sigma();
size_t multi_tile_count(long long nnz);   // tiles of one matrix (1 when nnz == 0)
size_t multi_mat_bytes();
void fill_multi_mat(void *dst, const void *val, const int *rowptr, const int *col,
                    const double *x, double *y, long long nnz, int m, int tile0, int part_off,
                    double alpha, double beta, int val_kind);
int launch_multi_tile_spmv(const MultiTileLaunch &L, int val_kind, cudaStream_t stream);
// The tile partition of one matrix into part[0 .. ntiles] (nnz > 0).
int launch_tile_partition(int m, long long nnz, const int *rowptr, int sigma, int *part,
                          cudaStream_t stream);
// Configures (under lazy module loading: loads) every kernel of an FP64
// tile SpMV of shape sigma on the current device.
int tile_preload_f64(int sigma);
void set_wait_limit_ns(unsigned long long ns);
void set_test_stall(int on);
int launch_tile_analyse(int m, long long nnz, const int *rowptr, int sigma, void *work,
                        cudaStream_t stream);

// Row-split kernel (one sub-warp per row; kernel version 1).
int launch_rowsplit_spmv(int m, int n, long long nnz, double alpha, const double *val,
                         const int *rowptr, const int *col, const double *x, double beta,
                         double *y, cudaStream_t stream);

// y[i] = beta * y[i] (beta == 0 writes exact zeros), for m == 0 / nnz == 0.
int launch_scale_y(int m, double beta, double *y, cudaStream_t stream);

// ---- format conversion (setup kernels) ------------------------------------
// Row-sorted COO row indices -> CSR row pointer (atomic-free boundary scan).
int launch_coo_rows_to_rowptr(int m, long long nnz, const int *coo_row, int *rowptr,
                              cudaStream_t stream);
// CSC -> CSR transpose (stable: columns ascending inside each row).
size_t csc_to_csr_workspace_bytes(int m, int n, long long nnz);
// CSR structure of A -> CSR structure of A^T plus the permutation of values.
size_t csr_transpose_workspace_bytes(int m, int n, long long nnz);
int launch_csr_transpose(int m, int n, long long nnz, const int *rowptr, const int *col,
                         int *t_rowptr, int *t_col, int *perm, void *work, size_t work_bytes,
                         cudaStream_t stream);
int launch_gather_values(long long nnz, int val_kind, const void *src, const int *perm, void *dst,
                         cudaStream_t stream);
// spMspV's x-zero filter: CSR of the nonzeros with x[col] != 0.
size_t csr_filter_x_workspace_bytes(long long nnz);
int launch_csr_filter_x(int m, long long nnz, const int *rowptr, const int *col,
                        const double *val, const double *x, int *orowptr, int *ocol,
                        double *oval, void *work, size_t work_bytes, cudaStream_t stream);
int launch_csc_to_csr(int m, int n, long long nnz, const double *csc_val,
                      const int *csc_colptr, const int *csc_row, double *csr_val,
                      int *csr_rowptr, int *csr_col, void *work, size_t work_bytes,
                      cudaStream_t stream);

// y = alpha*A*x + beta*y with A in CSC (atomic-free, deterministic):
// inspector (row-ordered structure + permutation + tile partition into
// `work`) and executor (values into row order + tile kernel).  staged: the
// inspector also builds the staging indices (an analysis reused for many
// products) and the executor moves values through them; inspector and
// executor must agree on it.  work: cscmv_workspace_bytes, 256-byte
// aligned; csc_tile_workspace: the tile workspace inside it (its status
// word).
size_t cscmv_workspace_bytes(int m, int n, long long nnz);
int launch_csc_analyse(int m, int n, long long nnz, const int *colptr, const int *rowidx,
                       void *work, size_t work_bytes, bool staged, cudaStream_t stream);
int launch_csc_bind_values(int m, int n, long long nnz, const double *val, void *work,
                           size_t work_bytes, bool staged, cudaStream_t stream);
int launch_cscmv_analysed(int m, int n, long long nnz, double alpha, const double *val,
                          const double *x, double beta, double *y, void *work,
                          size_t work_bytes, bool staged, cudaStream_t stream);
int launch_cscmv(int m, int n, long long nnz, double alpha, const double *val,
                 const int *colptr, const int *rowidx, const double *x, double beta, double *y,
                 void *work, size_t work_bytes, cudaStream_t stream);
void *csc_tile_workspace(void *work, int m, int n, long long nnz);
// Stable sort of COO entries by keys in [0, key_bound), carrying the other
// index and the value (bucket_sort.cuh passes).  Workspace:
// coo_sort_workspace_bytes.
size_t coo_sort_workspace_bytes(int key_bound, long long nnz);
int launch_coo_sort(int key_bound, long long nnz, const int *keys, const int *other,
                    const double *val, int *keys_out, int *other_out, double *val_out,
                    void *work, size_t work_bytes, cudaStream_t stream);
// out_i[p] = in_i[perm[p]], out_d[p] = in_d[perm[p]] (either output may be null).
int launch_gather(long long nnz, const int *perm, const int *in_i, int *out_i,
                  const double *in_d, double *out_d, cudaStream_t stream);

// ---- per-device resources used by the host (drop-in) entry points --------
constexpr int kPipeChunks = 4;   // chunks of the host-array entry points' copy/compute overlap
struct DeviceContext {
    int device = -1;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;   // host -> device copies overlapping the kernels
    cudaEvent_t ev[6] = {};
    cudaEvent_t chunk_ev[kPipeChunks + 1] = {};  // copies done (inputs, then each chunk)
};
// Returns the context of the current device (created on first use).
DeviceContext *device_context();

// Grow-only device scratch buffers owned by the context (slot 0..15).
void *device_scratch(int slot, size_t bytes);

int default_sigma_for(int m, long long nnz);
int csr5_sigma_for(int m, long long nnz);
int device_num_sms();

}  // namespace sblas
