// Hardware probes: the ceilings that bound an FP64 SpMV on this GPU.
//
//   sblas_probe_fp64    DFMA throughput with all 32 lanes active and with one
//                       lane active (the FP64 pipe's cost per warp
//                       instruction does not depend on the active lanes)
//   sblas_probe_gather  random 8-byte loads from a vector resident in L2
//                       (one per nonzero in CSR SpMV; each moves a 32-byte
//                       sector from L2 to the SM)
//   sblas_probe_gather_smem  the same with shared memory reserved per CTA (moves
//                       the shared-memory / L1 split of the SM)
//   sblas_probe_stream  streaming read bandwidth from HBM
//
// Diagnostics only (not on the SpMV path): they allocate and free their own
// buffers and synchronise the device.
#include <cstdio>

#include "sblas_internal.h"

namespace sblas {
namespace {

__global__ void probe_dfma_kernel(double *out, int iters, int active)
{
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
    double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
    const double b = 1.0000001, c = 1e-9;
    if ((int)(threadIdx.x & 31) < active) {
        for (int i = 0; i < iters; ++i) {
            a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
            a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

__global__ void probe_fill_idx(int *idx, long long n, int range)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        // integer hash of i (a fixed pseudo-random column per position)
        unsigned h = (unsigned)(i * 2654435761u) ^ 0x9e3779b9u;
        h ^= h >> 15;
        h *= 2246822519u;
        h ^= h >> 13;
        h *= 3266489917u;
        h ^= h >> 16;
        idx[i] = (int)(h % (unsigned)range);
    }
}

__global__ void probe_gather_kernel(const double *__restrict__ x, const int *__restrict__ idx,
                                    long long n, double *out)
{
    constexpr int U = 8;
    double acc = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x * U;
    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * U; i + U <= n;
         i += stride) {
        int id[U];
#pragma unroll
        for (int u = 0; u < U; ++u) id[u] = __ldcs(idx + i + u);
        double v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) v[u] = __ldg(x + id[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) acc += v[u];
    }
    if (acc == 1.2345) out[0] = acc;
}

__global__ void probe_stream_kernel(const double2 *__restrict__ p, size_t n2, double *out)
{
    // four independent 16-byte loads in flight per thread per iteration
    constexpr int U = 4;
    double acc = 0.0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (U - 1) * stride < n2; i += U * stride) {
        double2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) v[u] = __ldcs(p + i + u * stride);
#pragma unroll
        for (int u = 0; u < U; ++u) acc += v[u].x + v[u].y;
    }
    for (; i < n2; i += stride) {
        const double2 v = __ldcs(p + i);
        acc += v.x + v.y;
    }
    if (acc == 1.2345) out[0] = acc;
}

int sms_now()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

}  // namespace
}  // namespace sblas

using namespace sblas;

#define PROBE_TRY(expr)                                                                    \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            set_error(SBLAS_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_));            \
            rc = SBLAS_ERR_CUDA;                                                           \
            goto done;                                                                     \
        }                                                                                  \
    } while (0)

extern "C" {

int sblas_probe_fp64(double *warp_instr_per_s_full, double *warp_instr_per_s_one_lane)
{
    clear_error();
    int rc = SBLAS_OK;
    const int sms = sms_now(), blocks = sms * 8, threads = 256, iters = 4096;
    double *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f;
    const double winstr = (double)blocks * (threads / 32) * iters * 8;
    PROBE_TRY(cudaMalloc(&out, sizeof(double) * blocks * threads));
    PROBE_TRY(cudaEventCreate(&e0));
    PROBE_TRY(cudaEventCreate(&e1));
    for (int pass = 0; pass < 2; ++pass) {
        const int active = pass == 0 ? 32 : 1;
        probe_dfma_kernel<<<blocks, threads>>>(out, 64, active);
        PROBE_TRY(cudaEventRecord(e0));
        probe_dfma_kernel<<<blocks, threads>>>(out, iters, active);
        PROBE_TRY(cudaEventRecord(e1));
        PROBE_TRY(cudaEventSynchronize(e1));
        PROBE_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (pass == 0 && warp_instr_per_s_full) *warp_instr_per_s_full = winstr / (ms * 1e-3);
        if (pass == 1 && warp_instr_per_s_one_lane)
            *warp_instr_per_s_one_lane = winstr / (ms * 1e-3);
    }
done:
    if (out) cudaFree(out);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}

int sblas_probe_gather_smem(int range, int smem_per_cta, double *gathers_per_s,
                            int *ctas_per_sm)
{
    clear_error();
    if (range <= 0 || smem_per_cta < 0) {
        set_error(SBLAS_ERR_ARG, "range must be positive, smem_per_cta not negative");
        return SBLAS_ERR_ARG;
    }
    int rc = SBLAS_OK;
    const long long n = 64LL << 20;
    const int sms = sms_now();
    int occ = 0;
    double *x = nullptr, *out = nullptr;
    int *idx = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f;
    // the dynamic shared memory is reserved, not used: it only moves the
    // shared-memory / L1 split the driver picks for the launch
    PROBE_TRY(cudaFuncSetAttribute(probe_gather_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   smem_per_cta));
    PROBE_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, probe_gather_kernel, 256,
                                                            (size_t)smem_per_cta));
    if (occ < 1) {
        set_error(SBLAS_ERR_ARG, "no CTA of 256 threads fits with %d bytes of shared memory",
                  smem_per_cta);
        rc = SBLAS_ERR_ARG;
        goto done;
    }
    if (ctas_per_sm) *ctas_per_sm = occ;
    PROBE_TRY(cudaMalloc(&x, sizeof(double) * (size_t)range));
    PROBE_TRY(cudaMalloc(&idx, sizeof(int) * (size_t)n));
    PROBE_TRY(cudaMalloc(&out, sizeof(double)));
    PROBE_TRY(cudaMemset(x, 0, sizeof(double) * (size_t)range));
    PROBE_TRY(cudaEventCreate(&e0));
    PROBE_TRY(cudaEventCreate(&e1));
    probe_fill_idx<<<sms * 8, 256>>>(idx, n, range);
    probe_gather_kernel<<<sms * occ, 256, smem_per_cta>>>(x, idx, n, out);
    PROBE_TRY(cudaEventRecord(e0));
    probe_gather_kernel<<<sms * occ, 256, smem_per_cta>>>(x, idx, n, out);
    PROBE_TRY(cudaEventRecord(e1));
    PROBE_TRY(cudaEventSynchronize(e1));
    PROBE_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (gathers_per_s) *gathers_per_s = (double)n / (ms * 1e-3);
done:
    cudaFuncSetAttribute(probe_gather_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 0);
    if (x) cudaFree(x);
    if (idx) cudaFree(idx);
    if (out) cudaFree(out);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}

int sblas_probe_gather(int range, double *gathers_per_s)
{
    return sblas_probe_gather_smem(range, 0, gathers_per_s, nullptr);
}

int sblas_probe_stream(double *bytes_per_s)
{
    clear_error();
    int rc = SBLAS_OK;
    const size_t bytes = size_t(4) << 30;
    const int sms = sms_now();
    double *buf = nullptr, *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f, best = 1e30f;
    PROBE_TRY(cudaMalloc(&buf, bytes));
    PROBE_TRY(cudaMalloc(&out, sizeof(double)));
    PROBE_TRY(cudaMemset(buf, 0, bytes));
    PROBE_TRY(cudaEventCreate(&e0));
    PROBE_TRY(cudaEventCreate(&e1));
    for (int r = 0; r < 5; ++r) {
        PROBE_TRY(cudaEventRecord(e0));
        probe_stream_kernel<<<sms * 8, 256>>>(reinterpret_cast<const double2 *>(buf), bytes / 16,
                                              out);
        PROBE_TRY(cudaEventRecord(e1));
        PROBE_TRY(cudaEventSynchronize(e1));
        PROBE_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) best = ms;
    }
    if (bytes_per_s) *bytes_per_s = (double)bytes / (best * 1e-3);
done:
    if (buf) cudaFree(buf);
    if (out) cudaFree(out);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}

}  // extern "C"
