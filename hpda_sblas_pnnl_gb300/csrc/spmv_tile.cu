// nnz-balanced tile kernel for y = alpha*A*x + beta*y, A in CSR.
//
// This is the single-GPU form of the reference's nnz-balanced partition
// (src/dspmv_mgpu_v1.cu:120-152: split nnz evenly, find the rows holding the
// cut points, flag rows split by a cut, fix those rows up in the merge at
// :304-319) and of its CSR5 tiles (include/detail/cuda/csr5_spmv_cuda.h:
// per-tile segmented sums plus a carry "calibrate" pass).  The cut points are
// here CTA tiles of TILE = THREADS * SIGMA nonzeros and, inside a tile,
// per-thread chunks of SIGMA consecutive nonzeros.
//
// Design for GB300 (measured: the FP64 pipe retires ~1.57e10 warp
// instructions/s whatever the number of active lanes, i.e. ~0.5 T DFMA/s,
// while HBM delivers ~7 TB/s = ~0.55 T nonzeros/s at 12-13 B/nonzero):
//  * every thread runs exactly SIGMA fused multiply-adds with all 32 lanes
//    active; a row ending inside the chunk only costs integer work and a
//    shared-memory store (the running sum restarts with a select);
//  * the per-thread partial of the row crossing a chunk boundary ("tail") is
//    combined at CTA level: one warp reduces runs of equal rows lane-
//    sequentially (THREADS/32 adds per lane, work-efficient) and a 5-step
//    segmented shuffle scan joins runs crossing lanes; the thread that holds
//    the end of the row adds the result to its partial ("head") once;
//  * rows are finished in a coalesced epilogue (alpha/beta applied once per
//    row, nothing at all when alpha = 1 and beta = 0);
//  * the row crossing a tile boundary is finished by a tiny fix-up kernel
//    that adds the FP64 carries in a fixed order (no atomics: results are
//    bit-reproducible run to run);
//  * val/col tiles are streamed with 1-D bulk TMA (cp.async.bulk) into a
//    two-stage shared-memory ring (L2 evict-first), x is gathered with an L2
//    evict-last hint, grids are persistent (a multiple of the SM count).
#include <cstdio>
#include <climits>

#include "ptx.cuh"
#include "sblas_internal.h"

namespace sblas {

namespace {

constexpr int STAGES = 2;
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;  // 2 s per wait, then error flag

// Device error codes written to status[0].
constexpr int DEV_ERR_TIMEOUT = 1;

__host__ __device__ constexpr size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

template <int VK>
struct ValTraits;
template <>
struct ValTraits<VAL_F64> {
    using T = double;
    static constexpr int BYTES = 8;
};
template <>
struct ValTraits<VAL_F32> {
    using T = float;
    static constexpr int BYTES = 4;
};
template <>
struct ValTraits<VAL_PATTERN> {
    using T = float;  // unused
    static constexpr int BYTES = 0;
};

template <int THREADS, int SIGMA, int VK>
struct Layout {
    static constexpr int TILE = THREADS * SIGMA;
    static constexpr int RCAP = TILE + 2;       // rows (+2) of a tile that fit in smem
    static constexpr int RSLOT = (RCAP + 8 + 3) / 4 * 4;  // per-stage row-pointer slot,
                                                           // 16-byte multiple with slack
    static constexpr int VB = ValTraits<VK>::BYTES;
    static constexpr size_t VAL = 0;
    static constexpr size_t COL = align16(VAL + size_t(STAGES) * TILE * VB);
    static constexpr size_t RPTR = align16(COL + size_t(STAGES) * TILE * 4);
    static constexpr size_t META = align16(RPTR + size_t(STAGES) * RSLOT * 4);
    static constexpr size_t RVAL = align16(META + size_t(STAGES) * 4 * 4);
    static constexpr size_t TAILV = align16(RVAL + size_t(RCAP) * 8);
    static constexpr size_t CIN = TAILV + size_t(THREADS) * 8;
    static constexpr size_t TAILK = CIN + size_t(THREADS) * 8;
    static constexpr size_t HEADK = TAILK + size_t(THREADS) * 4;
    static constexpr size_t HEADV = align16(HEADK + size_t(THREADS) * 4);
    static constexpr size_t BAR = align16(HEADV + size_t(THREADS) * 8);
    static constexpr size_t TOTAL = BAR + STAGES * 8;
};

struct TileArgs {
    int m;
    int n;
    long long nnz;
    int ntiles;
    double alpha;
    double beta;
    const void *val;
    const int *rowptr;
    const int *col;
    const double *x;
    double *y;
    const int *row_part;  // [ntiles + 1]
    double *carry;        // [ntiles]
    int *status;          // [1]
    int use_tma;          // val and col 16-byte aligned: bulk copies
    int rp_tma;           // rowptr 16-byte aligned: bulk copies of its tile slices
};

// y epilogue for one finished row value v.
template <int AB>
__device__ __forceinline__ double finish_row(double v, double alpha, double beta,
                                             const double *yp)
{
    if (AB == 0) return v;                               // alpha = 1, beta = 0
    if (AB == 1) return alpha * v;                       // beta = 0
    return fma(alpha, v, beta * __ldg(yp));              // general
}

// Stages tile `tile` into stage `s` (one producer thread): its owned-row
// range (R0, R1) from the partition (passed in, prefetched by the caller),
// val and col by bulk copy, and the row-pointer slice rowptr[R0 .. R1+1] by
// bulk copy of its 16-byte-aligned superset (a few entries at the very end of
// the array by plain loads).  All completes on the stage's mbarrier.
template <int THREADS, int SIGMA, int VK>
__device__ __forceinline__ void issue_tile(const TileArgs &a, unsigned char *smem, int tile,
                                           int s, int R0, int R1, uint64_t pol)
{
    using L = Layout<THREADS, SIGMA, VK>;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::BAR) + s;
    int *meta = reinterpret_cast<int *>(smem + L::META) + 4 * s;
    int *rslot = reinterpret_cast<int *>(smem + L::RPTR) + size_t(s) * L::RSLOT;
    const long long tb = (long long)tile * L::TILE;
    const long long cnt = (a.nnz - tb < L::TILE) ? (a.nnz - tb) : L::TILE;
    uint32_t vbytes = 0, cbytes = 0, rbytes = 0;
    if (a.use_tma) {
        vbytes = (uint32_t)((cnt * L::VB) & ~15ll);
        cbytes = (uint32_t)((cnt * 4) & ~15ll);
    }
    const int nr = R1 - R0;
    const int fits = (nr + 2) <= L::RCAP;
    int base = R0;
    if (fits && a.rp_tma) {
        const int count = min(nr + 2, a.m - R0 + 1);   // rowptr[R0 .. R0+count-1]
        const int a0 = R0 & ~3;
        const int a1 = R0 + count;
        const int safe_end = (a.m + 1) & ~3;            // bulk copies stay inside rowptr
        const int t_end = max(a0, min((a1 + 3) & ~3, safe_end));
        base = a0;
        rbytes = (uint32_t)(t_end - a0) * 4u;
        for (int i = t_end; i < a1; ++i) rslot[i - a0] = __ldg(a.rowptr + i);
    }
    meta[0] = R0;
    meta[1] = R1;
    meta[2] = base;
    meta[3] = fits;
    ptx::mbar_arrive_expect_tx(bar, vbytes + cbytes + rbytes);   // release: meta, plain loads
    if (vbytes)
        ptx::bulk_g2s(smem + L::VAL + size_t(s) * L::TILE * L::VB,
                      static_cast<const unsigned char *>(a.val) + tb * L::VB, vbytes, bar, pol);
    if (cbytes)
        ptx::bulk_g2s(smem + L::COL + size_t(s) * L::TILE * 4, a.col + tb, cbytes, bar, pol);
    if (rbytes) ptx::bulk_g2s(rslot, a.rowptr + base, rbytes, bar, pol);
}

template <int THREADS, int SIGMA, int VK, int AB>
__global__ void __launch_bounds__(THREADS) tile_spmv_kernel(const TileArgs a)
{
    using L = Layout<THREADS, SIGMA, VK>;
    using VT = typename ValTraits<VK>::T;
    constexpr int TILE = L::TILE;
    constexpr int PER = THREADS / 32;  // tails reduced per lane in the carry pass

    extern __shared__ __align__(128) unsigned char smem[];
    VT *val_s = reinterpret_cast<VT *>(smem + L::VAL);
    int *col_s = reinterpret_cast<int *>(smem + L::COL);
    int *rptr_base = reinterpret_cast<int *>(smem + L::RPTR);
    const int *meta_s = reinterpret_cast<const int *>(smem + L::META);
    double *rval_s = reinterpret_cast<double *>(smem + L::RVAL);
    double *tailv_s = reinterpret_cast<double *>(smem + L::TAILV);
    double *cin_s = reinterpret_cast<double *>(smem + L::CIN);
    int *tailk_s = reinterpret_cast<int *>(smem + L::TAILK);
    int *headk_s = reinterpret_cast<int *>(smem + L::HEADK);
    double *headv_s = reinterpret_cast<double *>(smem + L::HEADV);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::BAR);

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const uint64_t pol_stream = ptx::policy_evict_first();
    const uint64_t pol_x = ptx::policy_evict_last();

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) ptx::mbar_init(bar + s, 1);
        ptx::fence_mbar_init();
    }
    for (int i = tid; i < L::RCAP; i += THREADS) rval_s[i] = 0.0;  // kept zero between tiles
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            const int t = blockIdx.x + s * gridDim.x;
            if (t < a.ntiles)
                issue_tile<THREADS, SIGMA, VK>(a, smem, t, s, __ldg(a.row_part + t),
                                               __ldg(a.row_part + t + 1), pol_stream);
        }
    }

    const double alpha = a.alpha, beta = a.beta;
    int it = 0;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x, ++it) {
        const int s = it % STAGES;
        const uint32_t parity = (uint32_t)((it / STAGES) & 1);
        const long long tb = (long long)tile * TILE;
        const int cnt_tile = (int)((a.nnz - tb < TILE) ? (a.nnz - tb) : TILE);
        VT *vst = val_s + size_t(s) * TILE;
        int *cst = col_s + size_t(s) * TILE;
        int *rptr_s = rptr_base + size_t(s) * L::RSLOT;
        // the producer prefetches the partition entries of the tile it will
        // stage after this one's data is consumed
        const int nt = tile + STAGES * (int)gridDim.x;
        int nR0 = 0, nR1 = 0;
        if (tid == 0 && nt < a.ntiles) {
            nR0 = __ldg(a.row_part + nt);
            nR1 = __ldg(a.row_part + nt + 1);
        }
        cin_s[tid] = 0.0;
        if (tid == 0) a.carry[tile] = 0.0;
        // ragged end of the tile (or everything, without TMA): plain loads
        {
            const int vdone = a.use_tma ? (int)(((long long)cnt_tile * L::VB & ~15ll) / (L::VB ? L::VB : 1)) : 0;
            const int cdone = a.use_tma ? (int)(((long long)cnt_tile * 4 & ~15ll) / 4) : 0;
            if (VK != VAL_PATTERN)
                for (int i = vdone + tid; i < cnt_tile; i += THREADS)
                    vst[i] = static_cast<const VT *>(a.val)[tb + i];
            for (int i = cdone + tid; i < cnt_tile; i += THREADS) cst[i] = __ldg(a.col + tb + i);
        }
        const bool arrived = ptx::mbar_wait_bounded(bar + s, parity, WAIT_LIMIT_NS);
        const int R0 = meta_s[4 * s + 0];
        const int R1 = meta_s[4 * s + 1];
        const int rbase = meta_s[4 * s + 2];
        const bool fits = meta_s[4 * s + 3] != 0;     // CTA-uniform
        const int nr = R1 - R0;                        // rows owned by this tile
        if (arrived && fits && !a.rp_tma) {
            const int nload = min(nr + 2, a.m - R0 + 1);
            for (int i = tid; i < nload; i += THREADS) rptr_s[i] = __ldg(a.rowptr + R0 + i);
        }
        // B1: tile data and row pointer visible; a timed-out wait anywhere in
        // the CTA stops the CTA (uniform decision)
        if (__syncthreads_or(!arrived)) {
            if (tid == 0) atomicExch(a.status, DEV_ERR_TIMEOUT);
            break;
        }

        // ---------------- per-thread chunk: SIGMA consecutive nonzeros ----------
        const int c0 = tid * SIGMA;                          // local offset in tile
        const int cnt = max(0, min(SIGMA, cnt_tile - c0));
        const int s0 = (int)(tb + c0);                       // global nnz index
        auto rp = [&](int r) -> int {                        // rowptr[r], r in [R0, R1+1]
            return fits ? rptr_s[r - rbase] : __ldg(a.rowptr + r);
        };
        double xv[SIGMA];
        int r0 = R0, rl = R0;      // rows of the chunk's first and last nonzero
        bool sb = false;           // the first row began before the chunk
        unsigned mask = 0;         // bit j: nonzero j of the chunk starts a new row
        bool slow = !fits;         // empty rows inside the chunk, or rows not in smem
        if (cnt > 0) {
            // issue every gather of the chunk first (one L2 round trip per
            // chunk instead of one per nonzero); the row search below runs
            // while they are in flight
            if (cnt == SIGMA) {
#pragma unroll
                for (int j = 0; j < SIGMA; ++j)
                    xv[j] = ptx::ldg_x_issue(a.x + cst[c0 + j], pol_x);
            } else {
#pragma unroll
                for (int j = 0; j < SIGMA; ++j)
                    xv[j] = ptx::ldg_x_issue(a.x + cst[c0 + (j < cnt ? j : 0)], pol_x);
            }
            // last row r in [R0, R1] with rowptr[r] <= s0
            int lo = R0, hi = min(R1, a.m - 1);
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (rp(mid) <= s0) lo = mid; else hi = mid - 1;
            }
            r0 = lo;
            sb = rp(r0) < s0;
            // row starts strictly inside the chunk -> boundary bits
            int rr = r0, nx = rp(r0 + 1);
            const int send = s0 + cnt;
            while (nx < send) {
                mask |= 1u << (nx - s0);
                const int n2 = rp(rr + 2);
                slow |= (n2 == nx);   // an empty row follows: general path
                ++rr;
                nx = n2;
            }
            rl = rr;
        }
        const bool warp_slow = __any_sync(0xffffffffu, slow);
        double sum = 0.0;
        int head_row = -1;
        double head_val = 0.0;
        if (cnt > 0 && !warp_slow) {
            // branch-free FMA chain: at a row start the running sum is stored
            // (the first segment to the thread's head slot when the row began
            // in an earlier chunk) and restarted with a select
            double *dst = sb ? &headv_s[tid] : &rval_s[r0 - R0];
            double *nxt = &rval_s[r0 + 1 - R0];
#pragma unroll
            for (int j = 0; j < SIGMA; ++j) {
                const bool b = (mask >> j) & 1u;
                if (b) *dst = sum;
                dst = b ? nxt : dst;
                nxt = b ? nxt + 1 : nxt;
                sum = b ? 0.0 : sum;
                if (j < cnt) {
                    if (VK == VAL_PATTERN) sum += xv[j];
                    else sum = fma((double)vst[c0 + j], xv[j], sum);
                }
            }
            if (sb && mask != 0u) {
                head_row = r0;
                head_val = headv_s[tid];
            }
        } else if (cnt > 0) {
            // general path: empty rows, or row pointer read from global memory
            int r = r0;
            int next = rp(r + 1);
            bool first_seg = true;
#pragma unroll
            for (int j = 0; j < SIGMA; ++j) {
                const int k = s0 + j;
                if (j < cnt && k == next) {
                    // row r ended at k-1: a head (row began in an earlier chunk)
                    // or a complete row; restart the running sum
                    if (first_seg && sb) {
                        head_row = r;
                        head_val = sum;
                    } else if (fits) {
                        rval_s[r - R0] = sum;
                    } else {
                        a.y[r] = finish_row<AB>(sum, alpha, beta, a.y + r);
                    }
                    first_seg = false;
                    sum = 0.0;
                    ++r;
                    next = rp(r + 1);
                    while (next <= k) {   // empty rows
                        ++r;
                        next = rp(r + 1);
                    }
                }
                if (j < cnt) {
                    if (VK == VAL_PATTERN) sum += xv[j];
                    else sum = fma((double)vst[c0 + j], xv[j], sum);
                }
            }
        }
        tailv_s[tid] = sum;
        tailk_s[tid] = (cnt > 0) ? rl : -1;   // -1: no data, never emitted
        headk_s[tid] = head_row;
        __syncthreads();  // B2: tails/heads published; stage s no longer read

        if (tid == 0 && nt < a.ntiles) {
            ptx::fence_proxy_async_smem();
            issue_tile<THREADS, SIGMA, VK>(a, smem, nt, s, nR0, nR1, pol_stream);
        }

        // ---------------- carry pass: reduce runs of tails (warp 0) ------------
        if (warp == 0) {
            auto emit = [&](int key, double total, int after) {
                if (key < 0) return;
                if (after < THREADS && headk_s[after] == key) {
                    cin_s[after] = total;                    // joins a head
                } else if (after >= THREADS && key == R1) {
                    a.carry[tile] = total;                   // continues in next tile
                } else if (fits) {
                    rval_s[key - R0] = total;                // complete row
                } else {
                    a.y[key] = finish_row<AB>(total, alpha, beta, a.y + key);
                }
            };
            const int base = lane * PER;
            double acc = 0.0;
            int prevk = tailk_s[base];
            const int fk = prevk;
            double af = 0.0;
            int f_after = base + PER;
            bool broke = false;
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int i = base + q;
                const int key = tailk_s[i];
                const bool brk = (q > 0) && (key != prevk);
                if (brk) {
                    if (!broke) {
                        af = acc;
                        f_after = i;
                        broke = true;
                    } else {
                        emit(prevk, acc, i);
                    }
                }
                acc = (brk ? 0.0 : acc) + tailv_s[i];
                prevk = key;
            }
            const bool single = !broke;
            const int kl = prevk;
            double S = acc;
            const int kl_prev = __shfl_up_sync(0xffffffffu, kl, 1);
            bool f = (lane == 0) || !single || (kl != kl_prev);
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const double So = __shfl_up_sync(0xffffffffu, S, d);
                const bool fo = __shfl_up_sync(0xffffffffu, f, d);
                const bool take = (lane >= d) && !f;
                S = S + (take ? So : 0.0);
                f = take ? fo : f;
            }
            const double S_prev = __shfl_up_sync(0xffffffffu, S, 1);
            // first run of a lane with several runs may continue from the left
            const double tot = af + ((lane > 0 && kl_prev == fk) ? S_prev : 0.0);
            if (!single) emit(fk, tot, f_after);
            // last run ends here unless the next lane starts with the same row
            const int next_first = (lane < 31) ? tailk_s[base + PER] : INT_MIN;
            if (lane == 31 || next_first != kl) emit(kl, S, base + PER);
        }
        __syncthreads();  // B3: carries in

        {   // head pass: every thread adds its carry-in once (converged add)
            const double hv = head_val + cin_s[tid];
            if (head_row >= 0) {
                if (fits) rval_s[head_row - R0] = hv;
                else a.y[head_row] = finish_row<AB>(hv, alpha, beta, a.y + head_row);
            }
        }
        __syncthreads();  // B4: row sums final

        if (fits) {
            // finished rows out (coalesced); the row-sum slots are cleared for
            // the next tile, which writes them only after its B1
            for (int i = tid; i < nr; i += THREADS) {
                a.y[R0 + i] = finish_row<AB>(rval_s[i], alpha, beta, a.y + R0 + i);
                rval_s[i] = 0.0;
            }
        } else {
            // rows without nonzeros were skipped above; write them here
            for (int rr = R0 + tid; rr < R1; rr += THREADS)
                if (__ldg(a.rowptr + rr) == __ldg(a.rowptr + rr + 1))
                    a.y[rr] = finish_row<AB>(0.0, alpha, beta, a.y + rr);
        }
    }

    // drain: a tile whose copies were issued but not consumed (early exit)
    if (tid == 0) {
        for (int k = 0; k < STAGES; ++k) {
            const int t = blockIdx.x + (it + k) * (int)gridDim.x;
            if (t < a.ntiles) {
                const int s = (it + k) % STAGES;
                ptx::mbar_wait_bounded(bar + s, (uint32_t)(((it + k) / STAGES) & 1),
                                       WAIT_LIMIT_NS);
            }
        }
    }
}

// part[k] = number of rows r with rowptr[r+1] <= k*TILE (k = 1..ntiles-1);
// part[0] = 0, part[ntiles] = m.  Row r is owned by the tile holding its
// last nonzero; empty rows by the tile holding the nonzero before them.
__global__ void tile_partition_kernel(int m, long long nnz, int ntiles, long long tile,
                                      const int *__restrict__ rowptr, int *__restrict__ part)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > ntiles) return;
    if (k == 0) { part[0] = 0; return; }
    if (k == ntiles) { part[k] = m; return; }
    const long long key = (long long)k * tile;
    // first i in [1, m] with rowptr[i] > key  ->  count = i - 1
    int lo = 1, hi = m;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((long long)__ldg(rowptr + mid) > key) hi = mid; else lo = mid + 1;
    }
    part[k] = lo - 1;
}

// Adds the carries of the tiles a row spans to the row, in tile order.
__global__ void tile_fixup_kernel(int ntiles, long long tile, double alpha,
                                  const int *__restrict__ rowptr, const int *__restrict__ part,
                                  const double *__restrict__ carry, double *__restrict__ y,
                                  const int *__restrict__ status)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (k >= ntiles) return;
    if (*status != 0) return;
    const int r = part[k];
    if (part[k + 1] <= r) return;                               // row r ends later
    if ((long long)__ldg(rowptr + r) >= (long long)k * tile) return;  // starts in tile k
    int j = k - 1;
    double c = carry[j];
    while (j >= 1 && part[j] == part[j + 1]) {
        c += carry[j - 1];
        --j;
    }
    y[r] = fma(alpha, c, y[r]);
}

__global__ void scale_y_kernel(int m, double beta, double *__restrict__ y)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        y[i] = (beta == 0.0) ? 0.0 : beta * y[i];
}

// ---------------- compiled shapes -----------------------------------------
constexpr int kThreads = 128;
constexpr int kSigmas[] = {7, 11, 15, 19, 23};
constexpr int kNumSigmas = sizeof(kSigmas) / sizeof(kSigmas[0]);

template <int SIGMA, int VK, int AB>
int launch_shape(const TileArgs &a, cudaStream_t stream)
{
    using L = Layout<kThreads, SIGMA, VK>;
    auto kfn = tile_spmv_kernel<kThreads, SIGMA, VK, AB>;
    static int configured_dev = -1;
    static int blocks_per_sm = 0;
    int dev = 0;
    SBLAS_CUDA_TRY(cudaGetDevice(&dev));
    if (configured_dev != dev) {
        SBLAS_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)L::TOTAL));
        int bps = 0;
        SBLAS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn, kThreads,
                                                                     L::TOTAL));
        if (bps < 1) {
            set_error(SBLAS_ERR_UNSUPPORTED, "tile shape sigma=%d does not fit on this GPU",
                      SIGMA);
            return SBLAS_ERR_UNSUPPORTED;
        }
        blocks_per_sm = bps;
        configured_dev = dev;
    }
    const int grid = min(a.ntiles, blocks_per_sm * device_num_sms());
    kfn<<<grid, kThreads, L::TOTAL, stream>>>(a);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

template <int SIGMA, int VK>
int launch_ab(const TileArgs &a, cudaStream_t stream)
{
    if (a.alpha == 1.0 && a.beta == 0.0) return launch_shape<SIGMA, VK, 0>(a, stream);
    if (a.beta == 0.0) return launch_shape<SIGMA, VK, 1>(a, stream);
    return launch_shape<SIGMA, VK, 2>(a, stream);
}

template <int SIGMA>
int launch_vk(int vk, const TileArgs &a, cudaStream_t stream)
{
    switch (vk) {
    case VAL_F64: return launch_ab<SIGMA, VAL_F64>(a, stream);
    case VAL_F32: return launch_ab<SIGMA, VAL_F32>(a, stream);
    case VAL_PATTERN: return launch_ab<SIGMA, VAL_PATTERN>(a, stream);
    default: break;
    }
    set_error(SBLAS_ERR_ARG, "unknown value kind %d", vk);
    return SBLAS_ERR_ARG;
}

}  // namespace

int tile_shape_count() { return kNumSigmas; }
TileShape tile_shape_at(int i) { return TileShape{kThreads, kSigmas[i]}; }
int tile_shape_index(int sigma)
{
    for (int i = 0; i < kNumSigmas; ++i)
        if (kSigmas[i] == sigma) return i;
    return -1;
}

static size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

size_t tile_workspace_bytes(long long nnz, int sigma)
{
    const long long tile = (long long)kThreads * sigma;
    const long long ntiles = (nnz + tile - 1) / tile;
    return align256(sizeof(int) * (size_t)(ntiles + 1)) + align256(sizeof(double) * (size_t)ntiles) +
           256;
}

int default_sigma_for(int m, long long nnz)
{
    (void)m;
    (void)nnz;
    return 19;
}

int csr5_sigma_for(int m, long long nnz)
{
    // include/anonymouslib_cuda.h:294-318: sigma from nonzeros per row
    // (<=4 -> 4, <=32 -> nnz/row, <=256 -> 32, else 6), mapped to the nearest
    // compiled (odd) shape.
    const long long per = m > 0 ? nnz / m : 0;
    const int want = per <= 4 ? 4 : (per <= 32 ? (int)per : (per <= 256 ? 32 : 6));
    int best = kSigmas[0], bd = 1 << 30;
    for (int i = 0; i < kNumSigmas; ++i) {
        const int d = kSigmas[i] > want ? kSigmas[i] - want : want - kSigmas[i];
        if (d < bd) {
            bd = d;
            best = kSigmas[i];
        }
    }
    return best;
}

int launch_scale_y(int m, double beta, double *y, cudaStream_t stream)
{
    if (m <= 0) return SBLAS_OK;
    const int threads = 256;
    const int blocks = min((m + threads - 1) / threads, 4 * device_num_sms());
    scale_y_kernel<<<blocks, threads, 0, stream>>>(m, beta, y);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

int launch_tile_analyse(int m, long long nnz, const int *rowptr, int sigma, void *work,
                        cudaStream_t stream)
{
    if (m <= 0 || nnz <= 0) return SBLAS_OK;
    if (tile_shape_index(sigma) < 0) {
        set_error(SBLAS_ERR_UNSUPPORTED, "sigma %d is not a compiled tile shape", sigma);
        return SBLAS_ERR_UNSUPPORTED;
    }
    const long long tile = (long long)kThreads * sigma;
    const long long ntiles_ll = (nnz + tile - 1) / tile;
    if (ntiles_ll > INT_MAX - 2) {
        set_error(SBLAS_ERR_ARG, "nnz %lld too large", nnz);
        return SBLAS_ERR_ARG;
    }
    const int ntiles = (int)ntiles_ll;
    int *part = static_cast<int *>(work);
    const int threads = 256;
    const int blocks = (ntiles + 1 + threads - 1) / threads;
    tile_partition_kernel<<<blocks, threads, 0, stream>>>(m, nnz, ntiles, tile, rowptr, part);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

int launch_tile_spmv(int m, int n, long long nnz, double alpha, const void *val, int val_kind,
                     const int *rowptr, const int *col, const double *x, double beta, double *y,
                     int sigma, void *work, cudaStream_t stream, bool analysed)
{
    if (m <= 0) return SBLAS_OK;
    if (nnz <= 0) return launch_scale_y(m, beta, y, stream);
    if (tile_shape_index(sigma) < 0) {
        set_error(SBLAS_ERR_UNSUPPORTED, "sigma %d is not a compiled tile shape", sigma);
        return SBLAS_ERR_UNSUPPORTED;
    }
    const long long tile = (long long)kThreads * sigma;
    const long long ntiles_ll = (nnz + tile - 1) / tile;
    if (ntiles_ll > INT_MAX - 2) {
        set_error(SBLAS_ERR_ARG, "nnz %lld too large", nnz);
        return SBLAS_ERR_ARG;
    }
    const int ntiles = (int)ntiles_ll;
    unsigned char *w = static_cast<unsigned char *>(work);
    int *part = reinterpret_cast<int *>(w);
    double *carry = reinterpret_cast<double *>(w + align256(sizeof(int) * (size_t)(ntiles + 1)));
    int *status = reinterpret_cast<int *>(w + align256(sizeof(int) * (size_t)(ntiles + 1)) +
                                          align256(sizeof(double) * (size_t)ntiles));
    SBLAS_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), stream));
    if (!analysed) {
        const int rc = launch_tile_analyse(m, nnz, rowptr, sigma, work, stream);
        if (rc != SBLAS_OK) return rc;
    }
    TileArgs a;
    a.m = m;
    a.n = n;
    a.nnz = nnz;
    a.ntiles = ntiles;
    a.alpha = alpha;
    a.beta = beta;
    a.val = val;
    a.rowptr = rowptr;
    a.col = col;
    a.x = x;
    a.y = y;
    a.row_part = part;
    a.carry = carry;
    a.status = status;
    const uintptr_t vb = reinterpret_cast<uintptr_t>(val), cb = reinterpret_cast<uintptr_t>(col);
    a.use_tma = ((val_kind == VAL_PATTERN || (vb & 15) == 0) && (cb & 15) == 0) ? 1 : 0;
    a.rp_tma = (reinterpret_cast<uintptr_t>(rowptr) & 15) == 0 ? 1 : 0;
    int rc = SBLAS_OK;
    switch (sigma) {
    case 7: rc = launch_vk<7>(val_kind, a, stream); break;
    case 11: rc = launch_vk<11>(val_kind, a, stream); break;
    case 15: rc = launch_vk<15>(val_kind, a, stream); break;
    case 19: rc = launch_vk<19>(val_kind, a, stream); break;
    case 23: rc = launch_vk<23>(val_kind, a, stream); break;
    default: rc = SBLAS_ERR_UNSUPPORTED; break;
    }
    if (rc != SBLAS_OK) return rc;
    if (ntiles > 1) {
        const int threads = 256;
        const int blocks = (ntiles - 1 + threads - 1) / threads;
        tile_fixup_kernel<<<blocks, threads, 0, stream>>>(ntiles, tile, alpha, rowptr, part, carry,
                                                         y, status);
        SBLAS_CUDA_TRY(cudaGetLastError());
    }
    return SBLAS_OK;
}

}  // namespace sblas
