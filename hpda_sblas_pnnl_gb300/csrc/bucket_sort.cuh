// Stable bucket scatter by one digit of an int key: the building block of
// this library's sorts (own kernels; no library sort).
//
// One pass over n entries, digit d(e) = (key(e) >> shift) & (nb - 1), nb <= 256:
//   bucket_hist_kernel    per CTA tile (TILE entries): digit counts (shared-
//                         memory counters), written digit-major: table[d * ntiles + t]
//   exclusive scan        of the table (scan_* kernels): entry (d, t) becomes the
//                         output position of tile t's first entry of digit d
//   bucket_scatter_kernel per tile: stable ranks of its entries (every warp walks
//                         its TILE / NW entries in order, ranking equal digits with
//                         a warp match and counting in a warp-private shared
//                         table), the tile sorted by digit in shared memory with
//                         its payloads, then written out so that consecutive
//                         threads write consecutive positions of one digit's run
//                         (about TILE / nb entries): coalesced stores.
//                         Every key and payload load of a tile is issued
//                         before the first is used, and tiles are small
//                         (~51 KB of shared memory, 64 registers per thread)
//                         so that four CTAs per SM hide the memory latency.
// Entries keep their input order inside every digit (tiles in order, warps in
// order inside a tile, entries in order inside a warp): a least-significant-
// digit sequence of passes is a stable sort.  Counts are integers and
// positions are computed, not claimed with atomics: every run produces the
// same output.
#pragma once

#include <climits>

#include "sblas_internal.h"

namespace sblas {
namespace bsort {
// internal linkage: every translation unit that includes this header gets its
// own copy of the kernels (no relocatable device code)
namespace {

constexpr int NW = 8;                   // warps per CTA
constexpr int THREADS = NW * 32;
constexpr int ITER = 8;                 // entries per lane per tile
constexpr int WSPAN = 32 * ITER;        // entries of one warp in a tile (256)
constexpr int TILE = NW * WSPAN;        // entries per CTA tile (2048)
constexpr int MAXB = 256;               // digit values per pass (8-bit digits)

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
// What an entry carries besides its key: up to two ints and one double.
struct Payload {
    int a;
    int b;
    double d;
};

// Op: __device__ int key(long long e) const: the sort key of entry e;
//     __device__ Payload load(State &st, long long e0, int lane, bool valid,
//                             long long e) const: entry e's payload, called by
//     all 32 lanes of a warp for the 32 consecutive entries e0 .. e0 + 31 (in
//     increasing e0 per warp, so Op::State may carry a cursor);
//     members key_out, a_out, b_out, d_out: the pass's outputs (a, b, d may
//     be null: not carried);
//     kPosOut: if true, the member pos_out receives every entry's output
//     position at its input index (pos_out[e] = position of e); the
//     payload's b must then be the entry's index e.
template <class Op>
__global__ void __launch_bounds__(THREADS, 4) bucket_scatter_kernel(const Op op, long long n,
                                                                 int shift, int nb, int ntiles,
                                                                 const int *__restrict__ table)
{
    extern __shared__ __align__(16) unsigned char bs_smem[];
    double *st_d = reinterpret_cast<double *>(bs_smem);                  // [TILE]
    int *st_key = reinterpret_cast<int *>(st_d + TILE);                  // [TILE]
    int *st_a = st_key + TILE;                                           // [TILE]
    int *st_b = st_a + TILE;                                             // [TILE]
    unsigned short *loc = reinterpret_cast<unsigned short *>(st_b + TILE);   // [TILE]
    unsigned short *wcnt = loc + TILE;                                   // [NW][MAXB]
    int *gbase = reinterpret_cast<int *>(wcnt + NW * MAXB);              // [MAXB]
    int *toff = gbase + MAXB;                                            // [MAXB]
    __shared__ int wtot[NW];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const long long t0 = (long long)blockIdx.x * TILE;
    const long long wbeg = t0 + (long long)w * WSPAN;
    const int cnt = (int)min((long long)TILE, n - t0);
    for (int i = tid; i < NW * MAXB; i += THREADS) wcnt[i] = 0;
    for (int d = tid; d < nb; d += THREADS)
        gbase[d] = __ldg(table + (long long)d * ntiles + blockIdx.x);
    // this warp's keys and payloads, every load in flight before the first
    // is used (the kernel is bound by memory latency otherwise)
    int kr[ITER];
    Payload pl[ITER];
    typename Op::State st{};
#pragma unroll
    for (int i = 0; i < ITER; ++i) {
        const long long e = wbeg + (long long)i * 32 + lane;
        kr[i] = e < n ? op.key(e) : 0;
    }
#pragma unroll
    for (int i = 0; i < ITER; ++i) {
        const long long e0 = wbeg + (long long)i * 32;
        pl[i] = (e0 < n) ? op.load(st, e0, lane, e0 + lane < n, e0 + lane)   // warp-uniform
                         : Payload{0, 0, 0.0};
    }
    __syncthreads();
    unsigned short *mycnt = wcnt + w * MAXB;
    const unsigned lt = (1u << lane) - 1u;
    // ranks: entries of this warp in order (batch i, then lane)
#pragma unroll
    for (int i = 0; i < ITER; ++i) {
        const long long e = wbeg + (long long)i * 32 + lane;
        const bool valid = e < n;
        const int d = valid ? digit_of(kr[i], shift, nb) : -1 - lane;   // invalid: unique
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
    // per digit: the warps' offsets inside the digit's run, the run lengths
    int total = 0;
    if (tid < nb) {
#pragma unroll
        for (int k = 0; k < NW; ++k) {
            const int c = wcnt[k * MAXB + tid];
            wcnt[k * MAXB + tid] = (unsigned short)total;
            total += c;
        }
    }
    // exclusive scan of the run lengths over the digits: each run's start in
    // the tile's sorted order (nb <= THREADS: one digit per thread)
    int v = total;
#pragma unroll
    for (int k = 1; k < 32; k <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, v, k);
        if (lane >= k) v += o;
    }
    if (lane == 31) wtot[w] = v;
    __syncthreads();
    int before = 0;
#pragma unroll
    for (int k = 0; k < NW; ++k) before += (k < w) ? wtot[k] : 0;
    if (tid < nb) toff[tid] = before + v - total;
    __syncthreads();
    // the tile in digit order, with its payloads, in shared memory
    const bool ha = op.a_out != nullptr, hd = op.d_out != nullptr;
    const bool hb = op.b_out != nullptr || Op::kPosOut;
#pragma unroll
    for (int i = 0; i < ITER; ++i) {
        const long long e = wbeg + (long long)i * 32 + lane;
        if (e < n) {
            const int d = digit_of(kr[i], shift, nb);
            const int slot = toff[d] + mycnt[d] + loc[w * WSPAN + i * 32 + lane];
            st_key[slot] = kr[i];
            if (ha) st_a[slot] = pl[i].a;
            if (hb) st_b[slot] = pl[i].b;
            if (hd) st_d[slot] = pl[i].d;
        }
    }
    __syncthreads();
    // write-out: consecutive slots of one digit go to consecutive positions
    for (int j = tid; j < cnt; j += THREADS) {
        const int k = st_key[j];
        const int d = digit_of(k, shift, nb);
        const long long pos = (long long)gbase[d] + (j - toff[d]);
        if (op.key_out) op.key_out[pos] = k;
        if (ha) op.a_out[pos] = st_a[j];
        if (op.b_out) op.b_out[pos] = st_b[j];
        if (hd) op.d_out[pos] = st_d[j];
        if constexpr (Op::kPosOut) op.pos_out[st_b[j]] = (int)pos;   // inside the tile's span
    }
}

inline size_t scatter_smem_bytes()
{
    return (sizeof(double) + 3 * sizeof(int) + sizeof(unsigned short)) * TILE +
           sizeof(unsigned short) * NW * MAXB + 2 * sizeof(int) * MAXB;
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
// work: pass_work_bytes(n, nb) bytes.  Stream-ordered.
template <class Op>
int scatter_pass(const Op &op, long long n, int shift, int nb, void *work, cudaStream_t stream)
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
    // four CTAs per SM (~208 KB): the largest shared-memory carveout; this
    // kernel's loads stream, nothing it reads is reused through L1
    SBLAS_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                        (int)cudaSharedmemCarveoutMaxShared));
    kfn<<<(unsigned)nt, THREADS, smem, stream>>>(op, n, shift, nb, (int)nt, table);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

// ---- segment of an entry in a compressed pointer array --------------------
// ptr[0..nseg] (ptr[0] = 0, ptr[nseg] = entries, nondecreasing): the segment
// (column of CSC, row of CSR) of entry e is the largest s with ptr[s] <= e.
// A warp walking increasing batches e0 .. e0 + 31 keeps the segment of its
// last batch in `cur` (-1 before the first): every batch then loads the 32
// segment starts after it (coalesced) and each lane counts those <= its
// entry with a 5-step shuffle search; runs of more than 32 short or empty
// segments take further rounds.
struct SegCursor {
    int cur = -1;
};

__device__ __forceinline__ int segment_of(const int *__restrict__ ptr, int nseg, SegCursor &c,
                                          long long e0, int lane, bool valid, long long e)
{
    if (c.cur < 0) {
        int lo = 0, hi = nseg - 1;   // largest s with ptr[s] <= e0 (warp-uniform)
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((long long)__ldg(ptr + mid) <= e0) lo = mid; else hi = mid - 1;
        }
        c.cur = lo;
    }
    const int ev = valid ? (int)e : INT_MIN;   // invalid lanes are found at once
    int base = c.cur, seg = c.cur;
    bool found = !valid;
    for (;;) {
        const int idx = base + 1 + lane;
        const int st = idx <= nseg ? __ldg(ptr + idx) : INT_MAX;
        int pos = 0;   // number of the 32 starts <= ev
#pragma unroll
        for (int b = 16; b > 0; b >>= 1) {
            const int v = __shfl_sync(0xffffffffu, st, pos + b - 1);
            if (v <= ev) pos += b;
        }
        const int v31 = __shfl_sync(0xffffffffu, st, 31);
        if (pos == 31 && v31 <= ev) pos = 32;
        if (!found && pos < 32) {
            seg = base + pos;
            found = true;
        }
        if (__all_sync(0xffffffffu, found)) break;
        base += 32;
    }
    c.cur = __shfl_sync(0xffffffffu, valid ? seg : c.cur, 31);
    return seg < nseg ? seg : nseg - 1;   // a malformed pointer never indexes past it
}

// ---- operations of the sorts ------------------------------------------------
// Moves (key, a, b, d) from arrays to the pass's output positions; any of
// a, b, d may be absent (null input and output).
struct MoveOp {
    const int *key_in;
    const int *a_in;
    const int *b_in;
    const double *d_in;
    int *key_out;
    int *a_out;
    int *b_out;
    double *d_out;
    static constexpr bool kPosOut = false;
    struct State {};
    __device__ int key(long long e) const { return __ldg(key_in + e); }
    __device__ Payload load(State &, long long, int, bool valid, long long e) const
    {
        Payload p{0, 0, 0.0};
        if (valid) {
            if (a_in) p.a = __ldg(a_in + e);
            if (b_in) p.b = __ldg(b_in + e);
            if (d_in) p.d = __ldg(d_in + e);
        }
        return p;
    }
};

// A compressed matrix's entries keyed by their index array (CSC: the row of
// every entry), carrying the segment each entry belongs to (CSC: its column)
// as `a`, the entry's own position as `b` and its value as `d`, as the
// outputs ask.
struct SegmentOp {
    const int *key_in;
    const int *ptr;      // segment pointer, nseg + 1 entries
    int nseg;
    const double *d_in;  // values, or null
    int *key_out;
    int *a_out;          // segment of the entry, or null
    int *b_out;          // position of the entry, or null
    double *d_out;
    static constexpr bool kPosOut = false;
    struct State {
        SegCursor c;
    };
    __device__ int key(long long e) const { return __ldg(key_in + e); }
    __device__ Payload load(State &st, long long e0, int lane, bool valid, long long e) const
    {
        Payload p{0, (int)e, 0.0};
        if (a_out) p.a = segment_of(ptr, nseg, st.c, e0, lane, valid, e);
        if (valid && d_in) p.d = __ldg(d_in + e);
        return p;
    }
};

// Digit widths of a least-significant-digit sort of keys in [0, key_bound):
// as few passes as digits of at most 8 bits allow, equal widths.
struct LsdPlan {
    int passes;
    int width;
};
inline LsdPlan lsd_plan(long long key_bound)
{
    int bits = 1;
    while (bits < 31 && (1LL << bits) < key_bound) ++bits;
    const int passes = (bits + 7) / 8;
    return LsdPlan{passes, (bits + passes - 1) / passes};
}

}  // namespace
}  // namespace bsort
}  // namespace sblas
