// Device-pointer C ABI (include/sblas_gb300.h), error state and per-device
// context of libsblas_gb300.so.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "sblas_internal.h"

namespace sblas {

namespace {
thread_local char g_msg[512] = "";
thread_local int g_status = SBLAS_OK;
int g_compat = -1;  // -1: not read from the environment yet
std::mutex g_ctx_mu;
constexpr int kMaxDevices = 64;
DeviceContext g_ctx[kMaxDevices];
struct Scratch {
    void *p = nullptr;
    size_t bytes = 0;
};
Scratch g_scratch[kMaxDevices][16];
}  // namespace

void set_error(int code, const char *fmt, ...)
{
    g_status = code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
}

void clear_error()
{
    g_status = SBLAS_OK;
    g_msg[0] = '\0';
}

int last_status() { return g_status; }

int device_num_sms()
{
    DeviceContext *c = device_context();
    return (c && c->num_sms > 0) ? c->num_sms : 148;
}

DeviceContext *device_context()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    DeviceContext &c = g_ctx[dev];
    if (c.device == dev) return &c;
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    if (c.device == dev) return &c;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return nullptr;
    cudaStream_t st = nullptr, cst = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    if (cudaStreamCreateWithFlags(&cst, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    for (auto &e : c.ev)
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    for (auto &e : c.chunk_ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    c.num_sms = sms;
    c.stream = st;
    c.copy_stream = cst;
    c.device = dev;
    return &c;
}

void *device_scratch(int slot, size_t bytes)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices || slot < 0 ||
        slot >= 16)
        return nullptr;
    Scratch &s = g_scratch[dev][slot];
    if (bytes == 0) bytes = 256;
    if (s.bytes >= bytes) return s.p;
    if (s.p) {
        cudaDeviceSynchronize();
        cudaFree(s.p);
        s.p = nullptr;
        s.bytes = 0;
    }
    size_t want = bytes + bytes / 8;
    want = (want + 4095) & ~size_t(4095);
    if (cudaMalloc(&s.p, want) != cudaSuccess) {
        cudaGetLastError();
        s.p = nullptr;
        return nullptr;
    }
    s.bytes = want;
    return s.p;
}

}  // namespace sblas

using namespace sblas;

extern "C" {

const char *sblas_last_error(void) { return g_msg; }
int sblas_last_status(void) { return g_status; }
const char *sblas_version(void) { return "sblas-gb300 0.1 (sm_103a)"; }

int sblas_stream_status(void *stream, int clear)
{
    clear_error();
    int word = 0;
    const int rc = tile_sticky_status(static_cast<cudaStream_t>(stream), clear != 0, &word);
    if (rc != SBLAS_OK) return rc;
    if (word != 0) {
        set_error(SBLAS_ERR_TIMEOUT,
                  "a tile kernel gave up a bounded wait (device word %d); its y is partial", word);
        return SBLAS_ERR_TIMEOUT;
    }
    return SBLAS_OK;
}

void sblas_set_wait_limit_ns(unsigned long long ns) { set_wait_limit_ns(ns); }

void sblas_test_hold_producer(int on) { set_test_stall(on); }

void sblas_set_compat_mode(int mode) { g_compat = mode ? 1 : 0; }

int sblas_get_compat_mode(void)
{
    if (g_compat < 0) {
        const char *e = getenv("SBLAS_COMPAT");
        g_compat = (e && strcmp(e, "reference") == 0) ? 1 : 0;
    }
    return g_compat;
}

size_t sblas_tile_workspace_bytes(long long nnz, int sigma)
{
    if (sigma <= 0) sigma = default_sigma_for(0, nnz);
    return tile_workspace_bytes(nnz, sigma);
}

int sblas_tile_sigma_count(void) { return tile_shape_count(); }
int sblas_tile_sigma_at(int i)
{
    return (i >= 0 && i < tile_shape_count()) ? tile_shape_at(i).sigma : -1;
}
int sblas_default_sigma(int m, long long nnz) { return default_sigma_for(m, nnz); }
int sblas_csr5_sigma(int m, long long nnz) { return csr5_sigma_for(m, nnz); }

int sblas_dcsrmv(int kernel, int m, int n, long long nnz, double alpha, const void *val,
                 int val_kind, const int *rowptr, const int *col, const double *x, double beta,
                 double *y, int sigma, void *work, size_t work_bytes, void *stream)
{
    clear_error();
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d n=%d nnz=%lld", m, n, nnz);
        return SBLAS_ERR_ARG;
    }
    if (kernel < 1 || kernel > 3) {
        set_error(SBLAS_ERR_ARG, "kernel must be 1, 2 or 3 (got %d)", kernel);
        return SBLAS_ERR_ARG;
    }
    if (val_kind < SBLAS_VAL_F64 || val_kind > SBLAS_VAL_PATTERN) {
        set_error(SBLAS_ERR_ARG, "unknown value kind %d", val_kind);
        return SBLAS_ERR_ARG;
    }
    if (m == 0) return SBLAS_OK;
    if (y == nullptr || (nnz > 0 && (rowptr == nullptr || col == nullptr || x == nullptr ||
                                     (val_kind != SBLAS_VAL_PATTERN && val == nullptr)))) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    if (kernel == 1) {
        if (val_kind != SBLAS_VAL_F64) {
            set_error(SBLAS_ERR_UNSUPPORTED, "kernel 1 takes FP64 values only");
            return SBLAS_ERR_UNSUPPORTED;
        }
        return launch_rowsplit_spmv(m, n, nnz, alpha, static_cast<const double *>(val), rowptr,
                                    col, x, beta, y, st);
    }
    if (sigma <= 0)
        sigma = (kernel == SBLAS_KERNEL_CSR5) ? csr5_sigma_for(m, nnz) : default_sigma_for(m, nnz);
    const size_t need = tile_workspace_bytes(nnz, sigma);
    if (work == nullptr) {
        work = device_scratch(0, need);
        if (!work) {
            set_error(SBLAS_ERR_ALLOC, "cannot allocate %zu bytes of workspace", need);
            return SBLAS_ERR_ALLOC;
        }
    } else if (work_bytes < need || (reinterpret_cast<uintptr_t>(work) & 255) != 0) {
        set_error(SBLAS_ERR_ARG, "workspace needs %zu bytes at 256-byte alignment", need);
        return SBLAS_ERR_ARG;
    }
    return launch_tile_spmv(m, n, nnz, alpha, val, val_kind, rowptr, col, x, beta, y, sigma,
                            work, st);
}

int sblas_csr_analyse(int kernel, int m, long long nnz, const int *rowptr, int sigma, void *work,
                      size_t work_bytes, void *stream)
{
    clear_error();
    if (m < 0 || nnz < 0 || nnz > 0x7fffffffLL || kernel < 2 || kernel > 3 || work == nullptr) {
        set_error(SBLAS_ERR_ARG, "sblas_csr_analyse: bad arguments");
        return SBLAS_ERR_ARG;
    }
    if (sigma <= 0)
        sigma = (kernel == SBLAS_KERNEL_CSR5) ? csr5_sigma_for(m, nnz) : default_sigma_for(m, nnz);
    if (work_bytes < tile_workspace_bytes(nnz, sigma) ||
        (reinterpret_cast<uintptr_t>(work) & 255) != 0) {
        set_error(SBLAS_ERR_ARG, "workspace needs %zu bytes at 256-byte alignment",
                  tile_workspace_bytes(nnz, sigma));
        return SBLAS_ERR_ARG;
    }
    return launch_tile_analyse(m, nnz, rowptr, sigma, work, static_cast<cudaStream_t>(stream));
}

int sblas_dcsrmv_analysed(int kernel, int m, int n, long long nnz, double alpha, const void *val,
                          int val_kind, const int *rowptr, const int *col, const double *x,
                          double beta, double *y, int sigma, void *work, size_t work_bytes,
                          void *stream)
{
    clear_error();
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL || kernel < 2 || kernel > 3 ||
        work == nullptr || val_kind < SBLAS_VAL_F64 || val_kind > SBLAS_VAL_PATTERN) {
        set_error(SBLAS_ERR_ARG, "sblas_dcsrmv_analysed: bad arguments");
        return SBLAS_ERR_ARG;
    }
    if (m == 0) return SBLAS_OK;
    if (y == nullptr || (nnz > 0 && (rowptr == nullptr || col == nullptr || x == nullptr ||
                                     (val_kind != SBLAS_VAL_PATTERN && val == nullptr)))) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    if (sigma <= 0)
        sigma = (kernel == SBLAS_KERNEL_CSR5) ? csr5_sigma_for(m, nnz) : default_sigma_for(m, nnz);
    if (work_bytes < tile_workspace_bytes(nnz, sigma) ||
        (reinterpret_cast<uintptr_t>(work) & 255) != 0) {
        set_error(SBLAS_ERR_ARG, "workspace needs %zu bytes at 256-byte alignment",
                  tile_workspace_bytes(nnz, sigma));
        return SBLAS_ERR_ARG;
    }
    return launch_tile_spmv(m, n, nnz, alpha, val, val_kind, rowptr, col, x, beta, y, sigma, work,
                            static_cast<cudaStream_t>(stream), true);
}

int sblas_dcoomv(int m, int n, long long nnz, double alpha, const double *val,
                 const int *coo_row, const int *coo_col, const double *x, double beta,
                 double *y, int *rowptr_work, int sigma, void *work, size_t work_bytes,
                 void *stream)
{
    clear_error();
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL || rowptr_work == nullptr) {
        set_error(SBLAS_ERR_ARG, "bad arguments");
        return SBLAS_ERR_ARG;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = launch_coo_rows_to_rowptr(m, nnz, coo_row, rowptr_work, st);
    if (rc != SBLAS_OK) return rc;
    return sblas_dcsrmv(SBLAS_KERNEL_MERGEPATH, m, n, nnz, alpha, val, SBLAS_VAL_F64,
                        rowptr_work, coo_col, x, beta, y, sigma, work, work_bytes, stream);
}

size_t sblas_csc_to_csr_workspace_bytes(int m, int n, long long nnz)
{
    return csc_to_csr_workspace_bytes(m, n, nnz);
}

int sblas_csc_to_csr(int m, int n, long long nnz, const double *csc_val, const int *csc_colptr,
                     const int *csc_row, double *csr_val, int *csr_rowptr, int *csr_col,
                     void *work, size_t work_bytes, void *stream)
{
    clear_error();
    return launch_csc_to_csr(m, n, nnz, csc_val, csc_colptr, csc_row, csr_val, csr_rowptr,
                             csr_col, work, work_bytes, static_cast<cudaStream_t>(stream));
}

size_t sblas_cscmv_workspace_bytes(int m, int n, long long nnz)
{
    return cscmv_workspace_bytes(m, n, nnz);
}

int sblas_dcscmv(int m, int n, long long nnz, double alpha, const double *val, const int *colptr,
                 const int *rowidx, const double *x, double beta, double *y, void *work,
                 size_t work_bytes, void *stream)
{
    clear_error();
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d n=%d nnz=%lld", m, n, nnz);
        return SBLAS_ERR_ARG;
    }
    if (m == 0) return SBLAS_OK;
    if (y == nullptr || (nnz > 0 && (val == nullptr || colptr == nullptr || rowidx == nullptr ||
                                     x == nullptr))) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    const size_t need = cscmv_workspace_bytes(m, n, nnz);
    if (work == nullptr) {
        work = device_scratch(14, need);
        work_bytes = need;
        if (!work) {
            set_error(SBLAS_ERR_ALLOC, "cannot allocate %zu bytes of workspace", need);
            return SBLAS_ERR_ALLOC;
        }
    }
    return launch_cscmv(m, n, nnz, alpha, val, colptr, rowidx, x, beta, y, work, work_bytes,
                        static_cast<cudaStream_t>(stream));
}

int sblas_csc_analyse(int m, int n, long long nnz, const int *colptr, const int *rowidx,
                      void *work, size_t work_bytes, void *stream)
{
    clear_error();
    if (nnz > 0 && (colptr == nullptr || rowidx == nullptr)) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    return launch_csc_analyse(m, n, nnz, colptr, rowidx, work, work_bytes, true,
                              static_cast<cudaStream_t>(stream));
}

int sblas_csc_bind_values(int m, int n, long long nnz, const double *val, void *work,
                          size_t work_bytes, void *stream)
{
    clear_error();
    if (nnz > 0 && val == nullptr) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    return launch_csc_bind_values(m, n, nnz, val, work, work_bytes, true,
                                  static_cast<cudaStream_t>(stream));
}

int sblas_dcscmv_analysed(int m, int n, long long nnz, double alpha, const double *val,
                          const double *x, double beta, double *y, void *work, size_t work_bytes,
                          void *stream)
{
    clear_error();
    if (m > 0 && (y == nullptr || (nnz > 0 && x == nullptr))) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    return launch_cscmv_analysed(m, n, nnz, alpha, val, x, beta, y, work, work_bytes, true,
                                 static_cast<cudaStream_t>(stream));
}

size_t sblas_csr_transpose_workspace_bytes(int m, int n, long long nnz)
{
    return csr_transpose_workspace_bytes(m, n, nnz);
}

int sblas_csr_transpose(int m, int n, long long nnz, const int *rowptr, const int *col,
                        int *t_rowptr, int *t_col, int *perm, void *work, size_t work_bytes,
                        void *stream)
{
    clear_error();
    if (t_rowptr == nullptr || (nnz > 0 && (rowptr == nullptr || col == nullptr ||
                                            t_col == nullptr || perm == nullptr))) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    return launch_csr_transpose(m, n, nnz, rowptr, col, t_rowptr, t_col, perm, work, work_bytes,
                                static_cast<cudaStream_t>(stream));
}

int sblas_gather_values(long long nnz, int val_kind, const void *src, const int *perm, void *dst,
                        void *stream)
{
    clear_error();
    if (nnz < 0 || (nnz > 0 && (src == nullptr || perm == nullptr || dst == nullptr))) {
        set_error(SBLAS_ERR_ARG, "bad size or null device pointer");
        return SBLAS_ERR_ARG;
    }
    return launch_gather_values(nnz, val_kind, src, perm, dst, static_cast<cudaStream_t>(stream));
}

size_t sblas_csr_filter_x_workspace_bytes(long long nnz)
{
    return csr_filter_x_workspace_bytes(nnz);
}

int sblas_csr_filter_x(int m, long long nnz, const int *rowptr, const int *col,
                       const double *val, const double *x, int *out_rowptr, int *out_col,
                       double *out_val, void *work, size_t work_bytes, void *stream)
{
    clear_error();
    if (rowptr == nullptr || out_rowptr == nullptr ||
        (nnz > 0 && (col == nullptr || x == nullptr || out_col == nullptr ||
                     (val == nullptr) != (out_val == nullptr)))) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    return launch_csr_filter_x(m, nnz, rowptr, col, val, x, out_rowptr, out_col, out_val, work,
                               work_bytes, static_cast<cudaStream_t>(stream));
}

int sblas_zero(void *p, size_t bytes, void *stream)
{
    clear_error();
    if (bytes == 0) return SBLAS_OK;
    if (p == nullptr) {
        set_error(SBLAS_ERR_ARG, "null device pointer");
        return SBLAS_ERR_ARG;
    }
    SBLAS_CUDA_TRY(cudaMemsetAsync(p, 0, bytes, static_cast<cudaStream_t>(stream)));
    return SBLAS_OK;
}

int sblas_coo_rows_to_rowptr(int m, long long nnz, const int *coo_row, int *rowptr,
                             void *stream)
{
    clear_error();
    return launch_coo_rows_to_rowptr(m, nnz, coo_row, rowptr, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
