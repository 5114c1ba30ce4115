// Row-split CSR kernel (kernel version 1).
//
// The reference's kernel 1 is cuSPARSE csrmv over an equal-row split
// (src/dspmv_mgpu_baseline.cu:64-70, :125-129).  Here one group of G lanes
// owns one row: the lanes stride over the row's nonzeros with FP64 FMAs,
// then reduce with shuffles.  G follows the mean row length (2..32).  This
// kernel is simple and exact but spends FP64 issue slots on idle lanes of
// short rows and on the shuffle reduction; the tile kernel (versions 2/3)
// is the fast path.
#include "sblas_internal.h"

namespace sblas {
namespace {

template <int G, int AB>
__global__ void __launch_bounds__(256) rowsplit_kernel(int m, double alpha, double beta,
                                                       const double *__restrict__ val,
                                                       const int *__restrict__ rowptr,
                                                       const int *__restrict__ col,
                                                       const double *__restrict__ x,
                                                       double *__restrict__ y)
{
    const int lane_g = threadIdx.x & (G - 1);
    const int groups = (gridDim.x * blockDim.x) / G;
    const unsigned mask = (G == 32) ? 0xffffffffu
                                    : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) / G; row < m; row += groups) {
        const int b = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
        double s = 0.0;
        for (int j = b + lane_g; j < e; j += G) s = fma(__ldg(val + j), __ldg(x + __ldg(col + j)), s);
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(mask, s, o, G);
        if (lane_g == 0) {
            if (AB == 0) y[row] = s;
            else if (AB == 1) y[row] = alpha * s;
            else y[row] = fma(alpha, s, beta * y[row]);
        }
    }
}

template <int G>
void launch_g(int m, double alpha, double beta, const double *val, const int *rowptr,
              const int *col, const double *x, double *y, cudaStream_t stream)
{
    const int threads = 256;
    const long long want = ((long long)m * G + threads - 1) / threads;
    const int blocks = (int)(want < 16LL * device_num_sms() ? want : 16LL * device_num_sms());
    if (alpha == 1.0 && beta == 0.0)
        rowsplit_kernel<G, 0><<<blocks, threads, 0, stream>>>(m, alpha, beta, val, rowptr, col, x, y);
    else if (beta == 0.0)
        rowsplit_kernel<G, 1><<<blocks, threads, 0, stream>>>(m, alpha, beta, val, rowptr, col, x, y);
    else
        rowsplit_kernel<G, 2><<<blocks, threads, 0, stream>>>(m, alpha, beta, val, rowptr, col, x, y);
}

}  // namespace

int launch_rowsplit_spmv(int m, int n, long long nnz, double alpha, const double *val,
                         const int *rowptr, const int *col, const double *x, double beta,
                         double *y, cudaStream_t stream)
{
    (void)n;
    if (m <= 0) return SBLAS_OK;
    if (nnz <= 0) return launch_scale_y(m, beta, y, stream);
    const double mean = (double)nnz / (double)m;
    if (mean <= 2.0) launch_g<2>(m, alpha, beta, val, rowptr, col, x, y, stream);
    else if (mean <= 4.0) launch_g<4>(m, alpha, beta, val, rowptr, col, x, y, stream);
    else if (mean <= 8.0) launch_g<8>(m, alpha, beta, val, rowptr, col, x, y, stream);
    else if (mean <= 16.0) launch_g<16>(m, alpha, beta, val, rowptr, col, x, y, stream);
    else launch_g<32>(m, alpha, beta, val, rowptr, col, x, y, stream);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

}  // namespace sblas
