/*
 * sblas_gb300.h -- device-pointer C ABI of libsblas_gb300.so.
 *
 * The drop-in entry points with the reference's signatures are declared in
 * spmv_kernel.h (host pointers, synchronous).  This header is the layer
 * under them: device pointers, a caller-supplied CUDA stream, asynchronous
 * and stream-ordered, no allocation inside a call unless stated.  It is what
 * the Python package (ctypes), CUDA-graph capture and batching use.
 *
 * Numerics: y = alpha * A * x + beta * y with A in CSR (int32 indices),
 * FP64 accumulation.  beta == 0 never reads y (NaNs in y are overwritten).
 * All functions return SBLAS_OK (0) or a negative status; the message of
 * the last failure on the calling thread is sblas_last_error().
 */
#ifndef SBLAS_GB300_H
#define SBLAS_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SBLAS_API __attribute__((visibility("default")))
#else
#define SBLAS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SBLAS_OK 0
#define SBLAS_ERR_ARG (-1)            /* invalid size, pointer or option */
#define SBLAS_ERR_NGPU (-2)           /* ngpu != 1: one GPU per process */
#define SBLAS_ERR_CUDA (-3)           /* a CUDA runtime call failed */
#define SBLAS_ERR_ALLOC (-4)          /* device allocation failed */
#define SBLAS_ERR_ALIGN (-5)          /* device array not 16-byte aligned */
#define SBLAS_ERR_KERNEL (-6)         /* a kernel reported a device-side error */
#define SBLAS_ERR_UNSUPPORTED (-7)    /* option not compiled in this build */
#define SBLAS_ERR_FORMAT (-8)         /* malformed input file (MatrixMarket reader) */
#define SBLAS_ERR_TIMEOUT (-9)        /* a kernel gave up a bounded wait; its output is partial */

/* kernel versions, numbered as the reference's `kernel` argument
 * (src/dspmv_mgpu_v1.cu:256-278) */
#define SBLAS_KERNEL_ROWSPLIT 1       /* one sub-warp per row */
#define SBLAS_KERNEL_MERGEPATH 2      /* nnz-balanced tiles, merge-path partition */
#define SBLAS_KERNEL_CSR5 3           /* nnz-balanced tiles, CSR5 sigma rule */

/* value storage of the matrix */
#define SBLAS_VAL_F64 0
#define SBLAS_VAL_F32 1               /* FP32 values, FP64 row sums */
#define SBLAS_VAL_PATTERN 2           /* binary matrix, no value array */

/* Message describing the last failure on this thread ("" if none). */
SBLAS_API const char *sblas_last_error(void);
/* Status code of the last call on this thread. */
SBLAS_API int sblas_last_status(void);
/* Library version string. */
SBLAS_API const char *sblas_version(void);

/* Device-side failures of the asynchronous entry points.  Every wait inside
 * the tile kernels is bounded (2 s by default); a launch that gives up a wait
 * stops early, leaves y partly written and records it in a sticky per-device
 * word.  This call waits for `stream` to complete, then returns SBLAS_OK or
 * SBLAS_ERR_TIMEOUT if any tile launch on the current device gave up a wait
 * since the word was last cleared (clear != 0 clears it).  The synchronous
 * entry points (spmv_kernel.h) check their own launches and return failure
 * themselves.  The reference has no counterpart: its checkCudaErrors prints
 * and exits (include/detail/cuda/helper_cuda.h:583-595). */
SBLAS_API int sblas_stream_status(void *stream, int clear);

/* Testing hooks (process-wide; not for production use).  The wait limit of
 * the tile kernels in nanoseconds (0 restores the default, 2 s), and a switch
 * that keeps the tile kernels' producer warp from staging any tile, so that
 * every launch's waits run out after the limit and report SBLAS_ERR_TIMEOUT:
 * the way tests exercise the failure path without faulting the GPU. */
SBLAS_API void sblas_set_wait_limit_ns(unsigned long long ns);
SBLAS_API void sblas_test_hold_producer(int on);

/* Reference-compatibility switches for the drop-in entry points (0 = off,
 * the default: every entry point computes y = alpha*A*x + beta*y on all rows).
 * 1 = reproduce the reference's observable results at ngpu = 1:
 *   - nnz-split entry points (v1, v1_numa*, v2) leave rows before the first
 *     and after the last non-empty row untouched;
 *   - the CSC entry points and v1_numa(_coo) with merg_opt = 0 add the result
 *     into the caller's y (y = y0 + alpha*A*x + beta*y0);
 *   - kernel 3 (CSR5) computes y = A*x, ignoring alpha and beta.
 * Process-wide; also set by the environment variable SBLAS_COMPAT=reference. */
SBLAS_API void sblas_set_compat_mode(int mode);
SBLAS_API int sblas_get_compat_mode(void);

/* Bytes of device workspace the tile kernels of sblas_dcsrmv need for nnz nonzeros with
 * tile parameter sigma (0 = library default). */
SBLAS_API size_t sblas_tile_workspace_bytes(long long nnz, int sigma);

/* Compiled tile shapes: sigma values usable below. */
SBLAS_API int sblas_tile_sigma_count(void);
SBLAS_API int sblas_tile_sigma_at(int i);
/* Default sigma chosen for a matrix shape (kernel 2), and the sigma of the
 * reference's CSR5 rule (kernel 3, include/anonymouslib_cuda.h:294-318). */
SBLAS_API int sblas_default_sigma(int m, long long nnz);
SBLAS_API int sblas_csr5_sigma(int m, long long nnz);

/*
 * y = alpha*A*x + beta*y, A in CSR on the device.  kernel: 1, 2 or 3.
 * val_kind: SBLAS_VAL_F64 (val is double*), SBLAS_VAL_F32 (float*) or
 * SBLAS_VAL_PATTERN (val ignored, every stored entry is 1.0); kernel 1 takes
 * FP64 values only.  sigma: nonzeros per thread of the tile kernels
 * (0 = default).  work/work_bytes: device workspace of at least
 * sblas_tile_workspace_bytes(nnz, sigma) bytes, 256-byte aligned, or NULL to
 * use a library-owned buffer (grown with cudaMalloc on first use; not
 * usable inside CUDA-graph capture).  stream: a cudaStream_t (0 = legacy
 * default stream).
 */
SBLAS_API int sblas_dcsrmv(int kernel, int m, int n, long long nnz, double alpha, const void *val,
                 int val_kind, const int *rowptr, const int *col, const double *x,
                 double beta, double *y, int sigma, void *work, size_t work_bytes,
                 void *stream);

/* Analysis / execution split of the tile kernels (kernel 2 or 3) for a
 * matrix used many times: sblas_csr_analyse writes the tile partition of the
 * row pointer into `work`; sblas_dcsrmv_analysed then runs only the tile
 * kernel and the carry fix-up, reusing it (same rowptr, nnz, sigma and
 * work).  Neither allocates, so both can be captured in a CUDA graph. */
SBLAS_API int sblas_csr_analyse(int kernel, int m, long long nnz, const int *rowptr, int sigma,
                                void *work, size_t work_bytes, void *stream);
SBLAS_API int sblas_dcsrmv_analysed(int kernel, int m, int n, long long nnz, double alpha,
                                    const void *val, int val_kind, const int *rowptr,
                                    const int *col, const double *x, double beta, double *y,
                                    int sigma, void *work, size_t work_bytes, void *stream);

/* Allocation-free FP64 CSR SpMV (the tile kernel, default tile shape) for
 * callers that cannot call cudaMalloc when they need it: code running inside
 * a device-memory pool or caching allocator, or services that reserve all
 * device memory at start-up and forbid allocation afterwards.  This entry
 * point has no counterpart in the reference.
 * Scratch: a fixed file-scope device array of sblas_noalloc_scratch_bytes()
 * bytes (7 MiB, held by every GPU that loads the library until exit); larger
 * matrices (about 0.86 G nonzeros and up) fail with SBLAS_ERR_ARG.  The
 * array is shared by every call: calls that overlap on the GPU race.  The
 * first call on a device resolves the array's address and creates the
 * library's per-device context (a stream and events); under CUDA's default
 * lazy module loading it is also when the library's module, and with it the
 * 7 MiB array, is placed in device memory (CUDA_MODULE_LOADING=EAGER places
 * it when the library loads).  A call with m = 0 does only that set-up:
 * make one before entering a region that forbids allocation, and before any
 * stream capture.  A bounded wait that gave up is reported by
 * sblas_stream_status.  Device arrays, stream-ordered on `stream`. */
SBLAS_API size_t sblas_noalloc_scratch_bytes(void);
SBLAS_API int sblas_dcsrmv_noalloc(int m, int n, int nnz, double alpha, const double *val,
                                   const int *rowptr, const int *col, const double *x,
                                   double beta, double *y, void *stream);

/* Row-sorted COO: builds the CSR row pointer on the device (atomic-free),
 * then runs the tile kernel.  rowptr_work: int[m + 1] device buffer. */
SBLAS_API int sblas_dcoomv(int m, int n, long long nnz, double alpha, const double *val,
                 const int *coo_row, const int *coo_col, const double *x, double beta,
                 double *y, int *rowptr_work, int sigma, void *work, size_t work_bytes,
                 void *stream);

/* CSC -> CSR on the device (stable; columns ascending inside each row): a
 * least-significant-digit bucket sort by row, 8-bit digits (three passes
 * up to 16M rows).
 * work: sblas_csc_to_csr_workspace_bytes(m, n, nnz) bytes. */
SBLAS_API size_t sblas_csc_to_csr_workspace_bytes(int m, int n, long long nnz);
SBLAS_API int sblas_csc_to_csr(int m, int n, long long nnz, const double *csc_val,
                     const int *csc_colptr, const int *csc_row, double *csr_val,
                     int *csr_rowptr, int *csr_col, void *work, size_t work_bytes,
                     void *stream);

/* y = alpha*A*x + beta*y with A in CSC on the device (colptr[n + 1],
 * rowidx[nnz], val[nnz]), the device form of spMV_mgpu_baseline_csc
 * (src/dspmv_mgpu_baseline_csc.cu:131-135 runs it as a transposed csrmv).
 * Inspector: a stable bucket sort of the entries by row gives A's row-ordered
 * structure and the permutation to it (sblas_csc_analyse, into `work`;
 * patterns above 2^20 entries also get staging indices); executor: the
 * values moved into row order (through L2-resident staging buckets after
 * sblas_csc_analyse; one direct gather in sblas_dcscmv) and the CSR tile
 * kernel (sblas_dcscmv_analysed, with the same work, colptr/rowidx
 * unchanged; val == NULL: the values last bound with sblas_csc_bind_values):
 * no atomics, bit-reproducible.  sblas_dcscmv runs both.  Rows need not be
 * sorted inside a column.  work: sblas_cscmv_workspace_bytes(m, n, nnz)
 * bytes, 256-byte aligned (sblas_dcscmv: or NULL for a library-owned
 * buffer).  A bounded wait that gave up is reported by sblas_stream_status. */
SBLAS_API size_t sblas_cscmv_workspace_bytes(int m, int n, long long nnz);
SBLAS_API int sblas_dcscmv(int m, int n, long long nnz, double alpha, const double *val,
                           const int *colptr, const int *rowidx, const double *x, double beta,
                           double *y, void *work, size_t work_bytes, void *stream);
SBLAS_API int sblas_csc_analyse(int m, int n, long long nnz, const int *colptr,
                                const int *rowidx, void *work, size_t work_bytes, void *stream);
SBLAS_API int sblas_dcscmv_analysed(int m, int n, long long nnz, double alpha, const double *val,
                                    const double *x, double beta, double *y, void *work,
                                    size_t work_bytes, void *stream);
/* Keeps `val` (CSC order) in row order inside the analysis in `work`;
 * sblas_dcscmv_analysed with val == NULL then uses these values and skips
 * the per-call gather (a CSR product's cost).  Bind again after the values
 * change. */
SBLAS_API int sblas_csc_bind_values(int m, int n, long long nnz, const double *val, void *work,
                                    size_t work_bytes, void *stream);

/* Row-sorted COO row indices -> CSR row pointer (int[m + 1]). */
SBLAS_API int sblas_coo_rows_to_rowptr(int m, long long nnz, const int *coo_row, int *rowptr,
                             void *stream);

/* ---- batched SpMM: many CSR matrices, k right-hand sides each ----------
 * Replaces the reference's multi-chunk task pool (spMV_mgpu_v2,
 * src/dspmv_mgpu_v2.cu:103-307, tasks include/spmv_task.h:4-36) on one GPU:
 * every matrix of the batch is cut into units of 32*s nonzeros and one
 * persistent kernel runs all units (then a short carry fix-up kernel).
 *   Y_i = alpha_i * A_i * X_i + beta_i * Y_i
 * X_i: n_i x k, row-major, row stride ldx >= k (the k values of one row
 * contiguous); Y_i: m_i x k, row-major, row stride ldy >= k.  For k >= 2, x
 * and y must be 16-byte aligned and ldx, ldy even.  k in {1, 2, 4, 8, 16};
 * s in {4, 8, 16, 32} (0: the default for k). */
typedef struct sblas_batch_matrix {
    int m;
    int n;
    long long nnz;          /* < 2^31 (int32 row pointer) */
    const void *val;        /* per val_kind; NULL for SBLAS_VAL_PATTERN */
    const int *rowptr;      /* m + 1 entries */
    const int *col;
    const double *x;
    int ldx;
    double *y;
    int ldy;
    double alpha;
    double beta;
    /* NULL, or m distinct row indices of Y (ascending): stored row r of the
     * matrix is row row_ids[r] of Y, and rows of Y not listed are left
     * untouched.  Lets a matrix with many empty rows be stored without them
     * (its row pointer then has one entry per listed row, plus one). */
    const int *row_ids;
    /* NULL, or nnz indices into val: stored entry p has value
     * val[val_perm[p]] (a transposed pattern reading the values of the
     * untransposed matrix, see sblas_csr_transpose). */
    const int *val_perm;
} sblas_batch_matrix;

typedef struct sblas_batch_plan sblas_batch_plan;

/* Default nonzeros per lane for k right-hand sides (0 if k not compiled). */
SBLAS_API int sblas_batch_default_s(int k);
/* Analysis: copies the descriptors to the device, computes the unit
 * partition and the persistent grid.  Allocates the plan's device memory
 * (descriptors, unit table, carries) and synchronises `stream`. */
SBLAS_API int sblas_batch_plan_create(int nmat, const sblas_batch_matrix *mats, int k,
                                      int val_kind, int s, void *stream,
                                      sblas_batch_plan **plan);
SBLAS_API int sblas_batch_plan_destroy(sblas_batch_plan *plan);
/* units of the plan, its s, and the device bytes it holds */
SBLAS_API int sblas_batch_plan_info(const sblas_batch_plan *plan, long long *units, int *s,
                                    size_t *device_bytes);
/* Runs the whole batch on `stream`: two kernel launches, no allocation, no
 * copy, no synchronisation (can be captured in a CUDA graph). */
SBLAS_API int sblas_batch_spmm(const sblas_batch_plan *plan, void *stream);
/* Single-matrix plans (nmat == 1): the same run with X, Y, alpha and beta
 * given per call (the structure and k fixed by the plan); val: values of
 * the plan's kind replacing the plan's (same pattern), or NULL. */
SBLAS_API int sblas_batch_spmm_xy(const sblas_batch_plan *plan, const void *val, const double *x,
                                  int ldx, double *y, int ldy, double alpha, double beta,
                                  void *stream);
/* Adjoint of Y = A X with respect to the stored values, for a single-matrix
 * plan: dval[p] = sum_c G[row(p), c] * X[col(p), c], p in CSR order.  G is
 * m x k (row stride ldg), X n x k; dval FP64 or FP32 as the plan's values
 * (pattern plans: SBLAS_ERR_UNSUPPORTED).  No counterpart in the reference. */
SBLAS_API int sblas_batch_sddmm(const sblas_batch_plan *plan, const double *g, int ldg,
                                const double *x, int ldx, void *dval, void *stream);

/* Transpose of a CSR structure on the device (setup for A^T products):
 * t_rowptr[n + 1], t_col[nnz] (the rows of A, ascending in each row of
 * A^T) and perm[nnz]: position in A of every entry of A^T, so that the
 * values of A^T are val[perm].  work: sblas_csr_transpose_workspace_bytes. */
SBLAS_API size_t sblas_csr_transpose_workspace_bytes(int m, int n, long long nnz);
SBLAS_API int sblas_csr_transpose(int m, int n, long long nnz, const int *rowptr, const int *col,
                                  int *t_rowptr, int *t_col, int *perm, void *work,
                                  size_t work_bytes, void *stream);
/* The x-zero filter of spMspV_mgpu_v1 / _v2 (src/dspmv_mgpu_v1.cu:29-40),
 * on the device: the nonzeros j with x[col[j]] != 0.0, in storage order, as
 * a CSR matrix out_rowptr[m + 1] (out_rowptr[m] = the kept count),
 * out_col / out_val (room for nnz entries).  val and out_val may both be
 * NULL (pattern).  rowptr[0] must be 0.  Asynchronous on stream; work:
 * sblas_csr_filter_x_workspace_bytes. */
SBLAS_API size_t sblas_csr_filter_x_workspace_bytes(long long nnz);
SBLAS_API int sblas_csr_filter_x(int m, long long nnz, const int *rowptr, const int *col,
                                 const double *val, const double *x, int *out_rowptr,
                                 int *out_col, double *out_val, void *work, size_t work_bytes,
                                 void *stream);
/* dst[p] = src[perm[p]] for nnz values of the given kind (FP64 or FP32). */
SBLAS_API int sblas_gather_values(long long nnz, int val_kind, const void *src, const int *perm,
                                  void *dst, void *stream);
/* ---- decomposition across devices (host code, no GPU) -------------------
 * The reference's nnz-balanced split of spMV_mgpu_v1 (src/dspmv_mgpu_v1.cu:
 * 120-152 cut points, :183-193 part row pointers, :304-319 merge) for a
 * caller that runs each part on its own device (one process per GPU) and
 * exchanges the parts' results itself.  Given the same per-part results the
 * merged y equals the reference's bit for bit. */
typedef struct sblas_nnz_part {
    int start_idx;    /* first nonzero of the part */
    int end_idx;      /* last nonzero of the part (inclusive, as the reference) */
    int start_row;    /* row holding start_idx */
    int end_row;      /* row holding end_idx */
    int start_flag;   /* 1: start_row begins in an earlier part (split row) */
    int end_flag;     /* 1: end_row continues in a later part */
    int m;            /* rows of the part: end_row - start_row + 1 */
    int nnz;          /* nonzeros of the part: end_idx - start_idx + 1 */
} sblas_nnz_part;

/* Cuts nnz = rowptr[m] nonzeros into nparts equal ranges (nnz >= nparts). */
SBLAS_API int sblas_nnz_partition(int m, long long nnz, const int *rowptr, int nparts,
                                  sblas_nnz_part *parts);
/* Row pointer of one part, part->m + 1 entries: 0, the inner rows rebased to
 * the part's first nonzero, part->nnz.  The part's columns and values are
 * col + start_idx and val + start_idx. */
SBLAS_API int sblas_part_rowptr(const int *rowptr, const sblas_nnz_part *part, int *out);
/* Merges the parts' results (part_y[d]: part d's m rows of
 * alpha*A_d*x + beta*y0) into y, which holds y0 on entry: rows copied in part
 * order, a split row gets the earlier parts' value added back and one
 * beta*y0 removed. */
SBLAS_API int sblas_merge_parts(int nparts, const sblas_nnz_part *parts,
                                const double *const *part_y, double beta, double *y);

/* Zero `bytes` bytes of device memory at p, stream-ordered (cudaMemsetAsync). */
SBLAS_API int sblas_zero(void *p, size_t bytes, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SBLAS_GB300_H */
