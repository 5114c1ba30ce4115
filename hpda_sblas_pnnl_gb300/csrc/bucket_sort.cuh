// Stable bucket scatter by one digit of an int key: the building block of
// this library's sorts and of the atomic-free CSC SpMV (own kernels; no
// library sort).
//
// One pass over n entries, digit d(e) = (key(e) >> shift) & (nb - 1), nb <= 2048:
//   bucket_hist_kernel   per CTA tile (TILE entries): digit counts (shared-memory
//                        counters), written bucket-major: table[d * ntiles + t]
//   exclusive scan       of the table (scan_* kernels): entry (d, t) becomes the
//                        output position of tile t's first entry of digit d
//   bucket_scatter_kernel per tile, stable ranks of its entries: every warp walks
//                        its TILE / NW entries in order, ranking equal digits with
//                        a warp match and counting in a warp-private shared table;
//                        a prefix over the warps per digit turns those counts into
//                        offsets; each entry then goes to
//                        scanned(d, t) + warp offset + rank, and the Op writes its
//                        payloads there.
// Entries keep their input order inside every digit (tiles in order, warps in
// order inside a tile, entries in order inside a warp): a least-significant-
// digit sequence of passes is a stable sort, and a single pass on the high
// bits groups entries into buckets in input order.  Counts are integers and
// positions are computed, not claimed with atomics: every run produces the
// same output.
#pragma once

#include <climits>

#include "sblas_internal.h"

namespace sblas {
namespace bsort {

constexpr int NW = 8;                   // warps per CTA
constexpr int THREADS = NW * 32;
constexpr int ITER = 64;                // entries per lane per tile
constexpr int WSPAN = 32 * ITER;        // entries of one warp in a tile (2048)
constexpr int TILE = NW * WSPAN;        // entries per CTA tile (16384)
constexpr int MAXB = 2048;              // digit values per pass

__host__ __device__ inline long long num_tiles(long long n) { return (n + TILE - 1) / TILE; }

__device__ __forceinline__ int digit_of(int key, int shift, int nb)
{
    return (int)(((unsigned)key >> shift) & (unsigned)(nb - 1));
}

// ---- pass 1: digit counts per tile ----------------------------------------
template <class Op>
__global__ void __launch_bounds__(THREADS) bucket_hist_kernel(const Op op, long long n, int shift,
                                                              int nb, int ntiles,
                                                              int *__restrict__ table)
{
    __shared__ int cnt[MAXB];
    for (int i = threadIdx.x; i < nb; i += THREADS) cnt[i] = 0;
    __syncthreads();
    const long long t0 = (long long)blockIdx.x * TILE;
    const int len = (int)min((long long)TILE, n - t0);
    for (int i = threadIdx.x; i < len; i += THREADS)
        atomicAdd(&cnt[digit_of(op.key(t0 + i), shift, nb)], 1);
    __syncthreads();
    for (int d = threadIdx.x; d < nb; d += THREADS)
        table[(long long)d * ntiles + blockIdx.x] = cnt[d];
}

// ---- exclusive scan of int counts (sums < 2^31) ---------------------------
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;   // 4096

// Exclusive scan of the CTA's SCAN_ITEMS values per thread (in registers,
// consecutive per thread); returns this thread's exclusive prefix and the
// CTA total in *total.
__device__ __forceinline__ int block_exclusive_prefix(int thread_sum, int *total)
{
    __shared__ int warp_tot[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v = thread_sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += o;
    }
    if (lane == 31) warp_tot[w] = v;
    __syncthreads();
    int wp = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < SCAN_THREADS / 32; ++k) {
        const int t = warp_tot[k];
        wp += (k < w) ? t : 0;
        tot += t;
    }
    __syncthreads();   // warp_tot may be reused by the caller's next call
    *total = tot;
    return wp + v - thread_sum;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_kernel(const int *__restrict__ in,
                                                                   long long n,
                                                                   int *__restrict__ sums)
{
    const long long base = (long long)blockIdx.x * SCAN_CHUNK;
    int s = 0;
    for (int i = threadIdx.x; i < SCAN_CHUNK; i += SCAN_THREADS)
        if (base + i < n) s += __ldg(in + base + i);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    __shared__ int ws[SCAN_THREADS / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < SCAN_THREADS / 32; ++k) t += ws[k];
        sums[blockIdx.x] = t;
    }
}

// One CTA: exclusive scan of the chunk sums in place (any count).
__global__ void __launch_bounds__(SCAN_THREADS) scan_sums_kernel(int *__restrict__ sums,
                                                                 int nchunks)
{
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nchunks; b0 += SCAN_CHUNK) {
        int v[SCAN_ITEMS];
        int ts = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            const int i = b0 + threadIdx.x * SCAN_ITEMS + k;
            v[k] = i < nchunks ? sums[i] : 0;
            ts += v[k];
        }
        int tot = 0;
        int p = block_exclusive_prefix(ts, &tot) + carry;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            const int i = b0 + threadIdx.x * SCAN_ITEMS + k;
            if (i < nchunks) sums[i] = p;
            p += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

// out[i] = sums[chunk] + exclusive prefix of in inside the chunk (in may
// alias out).  If total != nullptr, the last CTA writes the grand total there.
__global__ void __launch_bounds__(SCAN_THREADS) scan_apply_kernel(const int *in, long long n,
                                                                  const int *__restrict__ sums,
                                                                  int *out, int *total)
{
    const long long base = (long long)blockIdx.x * SCAN_CHUNK;
    int v[SCAN_ITEMS];
    int ts = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const long long i = base + threadIdx.x * SCAN_ITEMS + k;
        v[k] = i < n ? in[i] : 0;
        ts += v[k];
    }
    int tot = 0;
    int p = block_exclusive_prefix(ts, &tot) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const long long i = base + threadIdx.x * SCAN_ITEMS + k;
        if (i < n) out[i] = p;
        p += v[k];
    }
    if (total != nullptr && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
        *total = sums[blockIdx.x] + tot;
}

inline size_t scan_tmp_bytes(long long n)
{
    const long long chunks = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    return sizeof(int) * (size_t)(chunks > 0 ? chunks : 1);
}

// Exclusive scan of n ints (out may equal in); tmp: scan_tmp_bytes(n).
// total (device int*, may be null) receives the sum of all n values.
inline int exclusive_scan(const int *in, int *out, long long n, void *tmp, int *total,
                          cudaStream_t stream)
{
    if (n <= 0) {
        if (total) SBLAS_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(int), stream));
        return SBLAS_OK;
    }
    const long long chunks = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    if (chunks > INT_MAX) {
        set_error(SBLAS_ERR_ARG, "scan of %lld values too large", n);
        return SBLAS_ERR_ARG;
    }
    int *sums = static_cast<int *>(tmp);
    scan_reduce_kernel<<<(unsigned)chunks, SCAN_THREADS, 0, stream>>>(in, n, sums);
    scan_sums_kernel<<<1, SCAN_THREADS, 0, stream>>>(sums, (int)chunks);
    scan_apply_kernel<<<(unsigned)chunks, SCAN_THREADS, 0, stream>>>(in, n, sums, out, total);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

// ---- pass 2: stable scatter ------------------------------------------------
// Op: __device__ int key(long long e) const: the sort key of entry e;
//     __device__ void emit(State &st, long long e0, int lane, bool valid,
//                          long long e, int key, long long pos) const:
//     called by all 32 lanes of a warp for the 32 consecutive entries
//     e0 .. e0 + 31 (in increasing e0 per warp, so Op::State may carry a
//     cursor); writes entry e's outputs at position pos when valid.
template <class Op>
__global__ void __launch_bounds__(THREADS) bucket_scatter_kernel(const Op op, long long n,
                                                                 int shift, int nb, int ntiles,
                                                                 const int *__restrict__ table)
{
    extern __shared__ __align__(16) unsigned char bs_smem[];
    // wcnt[w][d]: counts, then each warp's offset inside the tile's run of d
    unsigned short *wcnt = reinterpret_cast<unsigned short *>(bs_smem);
    int *gbase = reinterpret_cast<int *>(bs_smem + sizeof(unsigned short) * NW * MAXB);
    unsigned short *loc = reinterpret_cast<unsigned short *>(
        bs_smem + sizeof(unsigned short) * NW * MAXB + sizeof(int) * MAXB);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long t0 = (long long)blockIdx.x * TILE;
    const long long wbeg = t0 + (long long)w * WSPAN;
    for (int i = threadIdx.x; i < NW * nb; i += THREADS) wcnt[(i / nb) * MAXB + (i % nb)] = 0;
    for (int d = threadIdx.x; d < nb; d += THREADS)
        gbase[d] = __ldg(table + (long long)d * ntiles + blockIdx.x);
    __syncthreads();
    unsigned short *mycnt = wcnt + w * MAXB;
    const unsigned lt = (1u << lane) - 1u;
    // ranks: entries of this warp in order (batch i, then lane)
    for (int i = 0; i < ITER; ++i) {
        const long long e = wbeg + (long long)i * 32 + lane;
        if (wbeg + (long long)i * 32 >= n) break;                  // warp-uniform
        const bool valid = e < n;
        const int d = valid ? digit_of(op.key(e), shift, nb) : -1 - lane;   // invalid: unique
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int base = valid ? (int)mycnt[d] : 0;
        __syncwarp();
        if (valid) {
            loc[w * WSPAN + i * 32 + lane] = (unsigned short)(base + __popc(peers & lt));
            if ((peers & lt) == 0u) mycnt[d] = (unsigned short)(base + __popc(peers));
        }
        __syncwarp();
    }
    __syncthreads();
    // per digit: warps' counts -> their offsets inside the tile's run
    for (int d = threadIdx.x; d < nb; d += THREADS) {
        int run = 0;
#pragma unroll
        for (int k = 0; k < NW; ++k) {
            const int c = wcnt[k * MAXB + d];
            wcnt[k * MAXB + d] = (unsigned short)run;
            run += c;
        }
    }
    __syncthreads();
    typename Op::State st{};
    for (int i = 0; i < ITER; ++i) {
        const long long e0 = wbeg + (long long)i * 32;
        if (e0 >= n) break;                                        // warp-uniform
        const long long e = e0 + lane;
        const bool valid = e < n;
        int key = 0;
        long long pos = 0;
        if (valid) {
            key = op.key(e);
            const int d = digit_of(key, shift, nb);
            pos = (long long)gbase[d] + mycnt[d] + loc[w * WSPAN + i * 32 + lane];
        }
        op.emit(st, e0, lane, valid, e, key, pos);
    }
}

inline size_t scatter_smem_bytes()
{
    return sizeof(unsigned short) * NW * MAXB + sizeof(int) * MAXB +
           sizeof(unsigned short) * TILE;
}

// Table bytes (counts / positions) and scan scratch of one pass over n entries.
inline size_t pass_table_bytes(long long n, int nb)
{
    return sizeof(int) * (size_t)nb * (size_t)(num_tiles(n) > 0 ? num_tiles(n) : 1);
}
inline size_t pass_work_bytes(long long n, int nb)
{
    const size_t t = (pass_table_bytes(n, nb) + 255) & ~size_t(255);
    return t + ((scan_tmp_bytes((long long)nb * num_tiles(n)) + 255) & ~size_t(255));
}

// One stable pass: entries of `op` scattered by digit (key >> shift) & (nb-1).
// work: pass_work_bytes(n, nb) bytes; on return the table holds, at
// [d * ntiles], the start of digit d's run for every d (and the runs end at
// n), stream-ordered.
template <class Op>
int scatter_pass(const Op &op, long long n, int shift, int nb, void *work, cudaStream_t stream,
                 int **table_out = nullptr)
{
    if (n <= 0) return SBLAS_OK;
    if (nb < 1 || nb > MAXB || (nb & (nb - 1)) != 0) {
        set_error(SBLAS_ERR_ARG, "bucket pass: %d buckets", nb);
        return SBLAS_ERR_ARG;
    }
    const long long nt = num_tiles(n);
    if (nt > INT_MAX / MAXB) {
        set_error(SBLAS_ERR_ARG, "bucket pass over %lld entries too large", n);
        return SBLAS_ERR_ARG;
    }
    int *table = static_cast<int *>(work);
    void *tmp = static_cast<unsigned char *>(work) + ((pass_table_bytes(n, nb) + 255) & ~size_t(255));
    static_assert(TILE <= 65536, "tile offsets are 16-bit");
    bucket_hist_kernel<Op><<<(unsigned)nt, THREADS, 0, stream>>>(op, n, shift, nb, (int)nt, table);
    SBLAS_CUDA_TRY(cudaGetLastError());
    const int rc = exclusive_scan(table, table, (long long)nb * nt, tmp, nullptr, stream);
    if (rc != SBLAS_OK) return rc;
    auto kfn = bucket_scatter_kernel<Op>;
    const size_t smem = scatter_smem_bytes();
    SBLAS_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
    kfn<<<(unsigned)nt, THREADS, smem, stream>>>(op, n, shift, nb, (int)nt, table);
    SBLAS_CUDA_TRY(cudaGetLastError());
    if (table_out) *table_out = table;
    return SBLAS_OK;
}

}  // namespace bsort
}  // namespace sblas
