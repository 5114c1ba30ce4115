// Batched CSR SpMM: many matrices of uneven size, K right-hand sides each,
// in one persistent launch (plus a short carry fix-up), the form the
// reference's task-pool schedule takes on one GPU
// (reference: src/dspmv_mgpu_v2.cu:103-307 hands nnz chunks of `nb` to a pool
// of streams; include/spmv_task.h:4-36 is the task record).
//
// Work unit: 32 * S consecutive nonzeros of one matrix, one warp.  Lane l
// owns nonzeros [U0 + l*S, U0 + l*S + S) and accumulates them sequentially in
// FP64 (K independent chains, one per right-hand side).  For every nonzero
// the K values of row col[j] of X are gathered as one contiguous 8K-byte
// piece (X row-major), so K right-hand sides cost one gather, not K.
//
// Rows:
//   - a row that starts and ends inside one lane's chunk goes to the warp's
//     row buffer in shared memory;
//   - a row crossing lanes: each lane keeps its last partial (tail) and its
//     first segment (head); the tails of a run of lanes are joined by direct
//     adds when every run spans at most four lanes, else by a segmented
//     shuffle scan; a unit lying inside one row is summed by a
//     reduce-scatter butterfly instead;
//   - a row crossing units: the unit's first-row partial (head) and
//     last-row partial (tail) go to per-unit carry arrays, and the fix-up
//     kernel adds, for every head, the tails of the preceding units of the
//     same row, in a fixed order (deterministic, no atomics);
//   - the unit's completed rows are written out by the whole warp at the
//     end (coalesced), alpha and beta applied once per row and column.
// Units with more rows than the row buffer holds, or with empty rows inside
// a chunk, take a per-lane general path with the same results.  Staged col
// and val sit at an odd per-lane stride (S + 1) so the lanes' strided
// shared-memory reads do not collide in a bank.  Matrices may list the rows
// of Y their stored rows write (row_ids) and read their values through a
// permutation (val_perm): the transposed operator of the adjoint uses both.
#pragma once

#include <climits>

#include "ptx.cuh"
#include "sblas_internal.h"

namespace sblas {
namespace batch {

constexpr int NW = 4;                 // warps per CTA
constexpr int CTA = NW * 32;

// device copy of one sblas_batch_matrix, plus its place in the unit list
struct Mat {
    const void *val;
    const int *rowptr;
    const int *col;
    const double *x;
    double *y;
    long long nnz;
    int m;
    int n;
    int ldx;
    int ldy;
    double alpha;
    double beta;
    int unit0;    // first unit of this matrix
    int nunits;   // units of this matrix (>= 1, also for nnz == 0)
    const int *row_ids;   // stored row r is row row_ids[r] of Y (nullptr: r)
    const int *val_perm;  // stored entry p has value val[val_perm[p]] (nullptr: val[p])
};

// row of Y that stored row r of a matrix writes
__device__ __forceinline__ long long out_row(const Mat *M, int r)
{
    return M->row_ids ? (long long)__ldg(M->row_ids + r) : (long long)r;
}

struct Args {
    const Mat *mats;
    int nmat;
    const int *unit_mat;   // [nunits] matrix of each unit
    const int *unit_row;   // [nunits] first row of each unit
    int *head_row;         // [nunits] row of the unit's head carry, -1: none
    double *head_val;      // [nunits * K]
    int *tail_row;         // [nunits] row of the unit's tail carry, -1: none
    double *tail_val;      // [nunits * K]
    int nunits;
    // single-matrix calls: X, Y, alpha, beta (and optionally the values)
    // given per call
    int override_xy;
    const double *x;
    double *y;
    int ldx;
    int ldy;
    double alpha;
    double beta;
    const void *val;       // nullptr: the plan's values
    // sampled product (adjoint of the values): dval[p] = G[row(p),:] . X[col(p),:]
    const double *g;
    int ldg;
    void *dval;            // FP64 or FP32 per the value kind
};

// Row stride (doubles) of the per-warp row and head buffers.  For K = 16 a
// row is 128 bytes, so the rows lanes store at the same time would all start
// in the same shared-memory bank: padded by two doubles.  Smaller K keep
// their stride (the padding would cost them a CTA per SM, which measured
// slower than the bank conflicts it removes).
template <int K>
constexpr int row_stride() { return K == 16 ? K + 2 : K; }

// CTAs of 128 threads per SM that the registers of a shape allow (ptxas:
// about 56-125 registers per thread for K = 1, 64 for K = 2, 80 for K = 4,
// 126 for K = 8, 216 for K = 16).  Used only to keep the shared memory of the
// resident CTAs within 196 KB per SM (rows_in_buffer); a stale entry costs
// speed, never correctness.
template <int K, int S>
constexpr int ctas_by_registers()
{
    return K == 1 ? (S == 4 ? 9 : S == 8 ? 8 : S == 16 ? 6 : 4)
                  : K == 2 ? 8 : K == 4 ? 6 : K == 8 ? 4 : 2;
}

constexpr size_t up16(size_t v) { return (v + 15) / 16 * 16; }

// Shared-memory bytes of one warp (WarpSmem below) for a row capacity r.
template <int K, int S, int VB>
constexpr size_t warp_smem_bytes(int r)
{
    const size_t staged = size_t(32 * S + 32);
    const size_t rp = up16(staged * 4 + staged * VB);
    const size_t rbuf = up16(rp + size_t(r + 2) * 4);
    return rbuf + size_t(r) * row_stride<K>() * 8 + size_t(32) * row_stride<K>() * 8;
}

// Rows of a unit held in the warp's row buffer: 8 S, at most 1536 / K; if
// the CTAs that fit on an SM would then need more than 196 KB of shared
// memory per SM (past that the driver takes the 228-KB carveout and random
// gathers run at less than half their rate), trimmed by up to a quarter
// until the same CTA count fits.
template <int K, int S, int VB>
constexpr int rows_in_buffer()
{
    constexpr size_t kLimit = size_t(195) * 1024;   // 196 KB less a 1-KB margin
    const int r = (8 * S < 1536 / K) ? 8 * S : 1536 / K;
    const size_t cta = 4 * warp_smem_bytes<K, S, VB>(r) + 1024;   // + the driver's 1 KB
    int occ = (int)(size_t(228 * 1024) / cta);
    if (occ > ctas_by_registers<K, S>()) occ = ctas_by_registers<K, S>();
    if (occ < 1 || (size_t)occ * cta <= kLimit) return r;
    const size_t budget = kLimit / occ - 1024;
    int t = r;
    while (t > r - r / 4 && 4 * warp_smem_bytes<K, S, VB>(t) > budget) --t;
    return 4 * warp_smem_bytes<K, S, VB>(t) <= budget ? t : r;
}

template <int K, int S, int VB>
struct Shape {
    static constexpr int UNIT = 32 * S;                        // nonzeros per unit
    static constexpr int RCAP = rows_in_buffer<K, S, VB>();    // rows in the buffer
    static constexpr int RPN = RCAP + 2;                       // row-pointer slice entries
};

template <int VK>
struct VT;
template <>
struct VT<VAL_F64> {
    using T = double;
    static constexpr int B = 8;
};
template <>
struct VT<VAL_F32> {
    using T = float;
    static constexpr int B = 4;
};
template <>
struct VT<VAL_PATTERN> {
    using T = float;   // unused
    static constexpr int B = 0;
};

// shared memory of one warp
template <int K, int S, int VK>
struct WarpSmem {
    using SH = Shape<K, S, VT<VK>::B>;
    static constexpr size_t COL = 0;
    // staged col and val: lane l's S entries at l*(S+1) (an odd stride for the
    // even S, so the lanes' strided reads hit different banks)
    static constexpr size_t VAL = COL + size_t(SH::UNIT + 32) * 4;
    static constexpr size_t RP = (VAL + size_t(SH::UNIT + 32) * VT<VK>::B + 15) / 16 * 16;
    static constexpr size_t RBUF = (RP + size_t(SH::RPN) * 4 + 15) / 16 * 16;
    static constexpr size_t HBUF = RBUF + size_t(SH::RCAP) * row_stride<K>() * 8;
    static constexpr size_t TOTAL = HBUF + size_t(32) * row_stride<K>() * 8;
};

template <int K, int S, int VK>
constexpr size_t cta_smem_bytes()
{
    static_assert(WarpSmem<K, S, VK>::TOTAL ==
                      warp_smem_bytes<K, S, VT<VK>::B>(Shape<K, S, VT<VK>::B>::RCAP),
                  "warp_smem_bytes follows WarpSmem");
    return size_t(NW) * WarpSmem<K, S, VK>::TOTAL;
}

// FP32 value widened to FP64 with integer operations (exact for every float
// class; the FP64 pipe stays free for the multiply-adds)
__device__ __forceinline__ double widen(float v)
{
    const unsigned u0 = __float_as_uint(v);
    const bool sub = (u0 & 0x7F800000u) == 0u && (u0 << 1) != 0u;
    const unsigned u = sub ? __float_as_uint(v * 0x1p64f) : u0;
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned ed = (e == 0xFFu) ? 0x7FFu : (e == 0u ? 0u : e + 896u - (sub ? 64u : 0u));
    const unsigned hi = (u & 0x80000000u) | (ed << 20) | ((u >> 3) & 0xFFFFFu);
    return __hiloint2double((int)hi, (int)(u << 29));
}

template <int VK>
__device__ __forceinline__ double value_at(const void *v)
{
    if constexpr (VK == VAL_F64) return *static_cast<const double *>(v);
    else if constexpr (VK == VAL_F32) return widen(*static_cast<const float *>(v));
    else return 1.0;
}

// K consecutive doubles of row c of X (16-byte aligned when K >= 2)
template <int K>
__device__ __forceinline__ void gather_row(const double *x, long long c, int ldx, double (&r)[K],
                                           uint64_t pol)
{
    const double *p = x + c * ldx;
    if constexpr (K == 1) {
        r[0] = ptx::ldg_x_issue(p, pol);
    } else {
#pragma unroll
        for (int q = 0; q < K / 2; ++q) {
            const double2 v = ptx::ldg_x2(reinterpret_cast<const double2 *>(p) + q, pol);
            r[2 * q] = v.x;
            r[2 * q + 1] = v.y;
        }
    }
}

template <int K>
__device__ __forceinline__ void store_row(double *dst, const double (&a)[K])
{
    if constexpr (K == 1) {
        dst[0] = a[0];
    } else {
#pragma unroll
        for (int q = 0; q < K / 2; ++q)
            reinterpret_cast<double2 *>(dst)[q] = make_double2(a[2 * q], a[2 * q + 1]);
    }
}

__device__ __forceinline__ double finish(double v, double alpha, double beta, const double *yp)
{
    return beta == 0.0 ? alpha * v : fma(alpha, v, beta * *yp);
}

// ---- main kernel: persistent, one warp per unit, units round-robin ---------
template <int K, int S, int VK>
__global__ void __launch_bounds__(CTA) batch_spmm_kernel(const Args a)
{
    using SH = Shape<K, S, VT<VK>::B>;
    using WS = WarpSmem<K, S, VK>;
    using T = typename VT<VK>::T;
    static_assert(S <= 32, "row-start mask is 32 bits");
    static_assert(K == 1 || K % 2 == 0, "K is 1 or even");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *ws = smem_raw + size_t(warp) * WS::TOTAL;
    int *scol = reinterpret_cast<int *>(ws + WS::COL);
    T *sval = reinterpret_cast<T *>(ws + WS::VAL);
    int *srp = reinterpret_cast<int *>(ws + WS::RP);
    double *rbuf = reinterpret_cast<double *>(ws + WS::RBUF);
    constexpr int KP = row_stride<K>();
    double *hbuf = reinterpret_cast<double *>(ws + WS::HBUF) + lane * KP;
    const uint64_t pol_x = ptx::policy_evict_last();
    const unsigned FULL = 0xffffffffu;

    for (int u = blockIdx.x * NW + warp; u < a.nunits; u += gridDim.x * NW) {
        const int b = __ldg(a.unit_mat + u);
        const Mat *M = a.mats + b;
        const int *rowptr = M->rowptr;
        const int *col = M->col;
        const void *val = (a.override_xy && a.val) ? a.val : M->val;
        const double *x = a.override_xy ? a.x : M->x;
        double *y = a.override_xy ? a.y : M->y;
        const int ldx = a.override_xy ? a.ldx : M->ldx;
        const int ldy = a.override_xy ? a.ldy : M->ldy;
        const double alpha = a.override_xy ? a.alpha : M->alpha;
        const double beta = a.override_xy ? a.beta : M->beta;
        // alpha and beta classified once per unit: a finished element costs
        // no FP64 operation for alpha = 1, beta = 0 (a compare of doubles
        // runs on the FP64 pipe too)
        const int abmode = (beta != 0.0) ? 2 : (alpha != 1.0) ? 1 : 0;
        auto fin = [&](double v, const double *yp) -> double {
            return abmode == 0 ? v : abmode == 1 ? alpha * v : fma(alpha, v, beta * *yp);
        };
        const int m = M->m;
        const int lu = u - M->unit0;
        const int U0 = lu * SH::UNIT;   // row pointers are int32: nnz < 2^31
        const int cntu = (int)min((long long)SH::UNIT, M->nnz - U0);
        const int RA = __ldg(a.unit_row + u);
        const int RB = (lu + 1 < M->nunits) ? __ldg(a.unit_row + u + 1) : m;
        const int nrows = RB - RA;
        const bool fits = nrows <= SH::RCAP;
        const int rp_hi = min(RB + 1, m);   // highest row-pointer index read

        // ---- stage the unit (coalesced), zero the row buffer ------------
        __syncwarp();
        for (int i = lane; i < cntu; i += 32) scol[i + i / S] = __ldcs(col + U0 + i);
        if constexpr (VK != VAL_PATTERN) {
            const T *vp = static_cast<const T *>(val);
            if (M->val_perm)
                for (int i = lane; i < cntu; i += 32)
                    sval[i + i / S] = __ldg(vp + __ldcs(M->val_perm + U0 + i));
            else
                for (int i = lane; i < cntu; i += 32) sval[i + i / S] = __ldcs(vp + U0 + i);
        }
        if (fits) {
            for (int i = lane; i <= rp_hi - RA; i += 32) srp[i] = __ldg(rowptr + RA + i);
            for (int i = lane; i < nrows * KP; i += 32) rbuf[i] = 0.0;
        }
        __syncwarp();
        auto rp = [&](int r) -> int { return fits ? srp[r - RA] : __ldg(rowptr + r); };

        // ---- this lane's chunk ------------------------------------------
        const int c0 = lane * S;            // first nonzero of the chunk in the unit
        const int cs0 = lane * (S + 1);     // its place in the staged col and val
        const int cnt = max(0, min(S, cntu - c0));
        const int s0 = U0 + c0, send = s0 + cnt;
        double xs[K == 1 ? S : 1];       // K == 1: every gather issued up front
        double cur[K];                   // K >= 2: one row of X ahead
        if (cnt > 0) {
            if constexpr (K == 1) {
#pragma unroll
                for (int j = 0; j < S; ++j)
                    xs[j] = ptx::ldg_x_issue(x + (long long)scol[cs0 + (j < cnt ? j : 0)] * ldx, pol_x);
            } else {
                gather_row<K>(x, scol[cs0], ldx, cur, pol_x);
            }
        }
        int r0 = RA, rl = RA;
        bool sb = false, ends = false, slow = !fits;
        unsigned mask = 0;
        if (cnt > 0) {
            int lo = RA, hi = min(RB, m - 1);
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (rp(mid) <= s0) lo = mid; else hi = mid - 1;
            }
            r0 = lo;
            sb = rp(r0) < s0;
            int rr = r0, nx = rp(r0 + 1);
            while (nx < send) {
                mask |= 1u << (nx - s0);
                const int n2 = rp(rr + 2);
                slow |= (n2 == nx);      // an empty row inside the chunk
                ++rr;
                nx = n2;
            }
            rl = rr;
            ends = (nx == send);
        }
        const bool warp_slow = __any_sync(FULL, slow);

        double acc[K];
#pragma unroll
        for (int c = 0; c < K; ++c) acc[c] = 0.0;
        bool has_head = false, has_tail = false, mid_lane = false;
        bool noemit = false;   // the chunk ends no row
        int hrow = -1, trow = -1;

        auto fma_row = [&](int j, const double (&xr)[K]) {
            const double v = value_at<VK>(sval + cs0 + j);
#pragma unroll
            for (int c = 0; c < K; ++c) {
                if constexpr (VK == VAL_PATTERN) acc[c] += xr[c];
                else acc[c] = fma(v, xr[c], acc[c]);
            }
        };
        auto step = [&](int j) {
            if constexpr (K == 1) {
                const double xr[1] = {xs[j]};
                fma_row(j, xr);
            } else {
                double nxt[K];
                if (j + 1 < cnt) gather_row<K>(x, scol[cs0 + j + 1], ldx, nxt, pol_x);
                fma_row(j, cur);
#pragma unroll
                for (int c = 0; c < K; ++c) cur[c] = nxt[c];
            }
        };

        if (cnt > 0 && !warp_slow) {
            // branch-free row emission: at a row start the running sums go to
            // the row buffer (or the head slot for a row begun before the
            // chunk) and restart
            double *dst = sb ? hbuf : rbuf + (r0 - RA) * KP;
            double *nxp = rbuf + (r0 + 1 - RA) * KP;
#pragma unroll
            for (int j = 0; j < S; ++j) {
                const bool bnd = (mask >> j) & 1u;
                if (bnd) store_row<K>(dst, acc);
                dst = bnd ? nxp : dst;
                nxp = bnd ? nxp + KP : nxp;
#pragma unroll
                for (int c = 0; c < K; ++c) acc[c] = bnd ? 0.0 : acc[c];
                if (j < cnt) step(j);
            }
            if (ends) store_row<K>(dst, acc);
            has_head = sb && (mask != 0u || ends);
            hrow = r0;
            has_tail = !ends;
            trow = rl;
            mid_lane = has_tail && sb && mask == 0u;
            noemit = mask == 0u && !ends;
        } else if (cnt > 0) {
            // general path: empty rows inside the chunk, or more rows than
            // the row buffer holds (rows then go straight to y)
            int r = r0, next = rp(r0 + 1);
            bool first = true;
            auto emit = [&](int row) {
                if (first && sb) {
                    store_row<K>(hbuf, acc);
                    has_head = true;
                    hrow = row;
                } else if (fits) {
                    store_row<K>(rbuf + (row - RA) * KP, acc);
                } else {
                    double *yr = y + out_row(M, row) * ldy;
#pragma unroll
                    for (int c = 0; c < K; ++c) yr[c] = fin(acc[c], yr + c);
                }
                first = false;
#pragma unroll
                for (int c = 0; c < K; ++c) acc[c] = 0.0;
            };
#pragma unroll
            for (int j = 0; j < S; ++j) {
                if (j < cnt) {
                    const int k = s0 + j;
                    if (next == k) {
                        emit(r);              // row r ends before nonzero k
                        ++r;
                        next = rp(r + 1);
                        while (next == k) {   // empty rows: written by the epilogue
                            ++r;
                            next = rp(r + 1);
                        }
                    }
                    step(j);
                }
            }
            if (next == send) {
                emit(r);
                ends = true;
            } else {
                has_tail = true;
                trow = r;
                mid_lane = first && sb;
                noemit = first;
            }
        }

        // ---- a unit inside one row that continues past it (every chunk full,
        // none ending a row): its total is the unit's tail carry, summed over
        // the lanes by a reduce-scatter butterfly (K - 1 + 5 - log2 K adds per
        // lane instead of the segmented scan's 5 K)
        if constexpr (K >= 2) {
            if (__all_sync(FULL, cnt == S && noemit)) {
                constexpr int LK = K == 2 ? 1 : K == 4 ? 2 : K == 8 ? 3 : 4;
                double v[K];
#pragma unroll
                for (int c = 0; c < K; ++c) v[c] = acc[c];
#pragma unroll
                for (int st = 0; st < LK; ++st) {
                    const int d = 16 >> st;
                    const int h = K >> (st + 1);
                    const bool up = (lane & d) != 0;
#pragma unroll
                    for (int i = 0; i < h; ++i) {
                        const double mine = up ? v[i + h] : v[i];
                        const double other = up ? v[i] : v[i + h];
                        v[i] = mine + __shfl_xor_sync(FULL, other, d);
                    }
                }
#pragma unroll
                for (int st = LK; st < 5; ++st) v[0] += __shfl_xor_sync(FULL, v[0], 16 >> st);
                if ((lane & ((1 << (5 - LK)) - 1)) == 0)
                    a.tail_val[(long long)u * K + (lane >> (5 - LK))] = v[0];
                if (lane == 0) {
                    a.tail_row[u] = trow;
                    a.head_row[u] = -1;
                }
                continue;   // no row of Y is finished in this unit
            }
        }

        // ---- rows crossing lanes: segmented scan of the tails -------------
        double sv[K];
#pragma unroll
        for (int c = 0; c < K; ++c) sv[c] = has_tail ? acc[c] : 0.0;
        if (!has_tail) trow = -1;
        const int trow_prev = __shfl_up_sync(FULL, trow, 1);
        const bool cont = mid_lane && lane > 0 && trow_prev == trow;
        const unsigned contm = __ballot_sync(FULL, cont);
        // run length: the consecutive lanes whose tails continue into this one
        const unsigned starts = ~contm & ((2u << lane) - 1u);
        const int lrun = contm ? lane - (31 - __clz(starts)) : 0;
        const int maxrun = contm ? __reduce_max_sync(FULL, (unsigned)lrun) : 0;
        if (maxrun > 0 && maxrun <= 3) {
            // short runs (the common case): add the few tails before each
            // lane directly, maxrun * K adds instead of the scan's 5 K
            double base[K];
#pragma unroll
            for (int c = 0; c < K; ++c) base[c] = sv[c];
#pragma unroll
            for (int d = 1; d <= 3; ++d) {
                if (d > maxrun) break;
#pragma unroll
                for (int c = 0; c < K; ++c) {
                    const double so = __shfl_up_sync(FULL, base[c], d);
                    sv[c] += (d <= lrun) ? so : 0.0;
                }
            }
        } else if (maxrun > 3) {
            bool f = !cont;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const bool fo = __shfl_up_sync(FULL, f, d);
                const bool take = (lane >= d) && !f;
#pragma unroll
                for (int c = 0; c < K; ++c) {
                    const double so = __shfl_up_sync(FULL, sv[c], d);
                    sv[c] += take ? so : 0.0;
                }
                f = take ? fo : f;
            }
        }
        double sprev[K];
#pragma unroll
        for (int c = 0; c < K; ++c) sprev[c] = __shfl_up_sync(FULL, sv[c], 1);
        const bool join = has_head && lane > 0 && trow_prev == hrow;
        const bool head_before_unit = has_head && hrow == RA && rp(RA) < U0;
        if (has_head) {
            double tot[K];
#pragma unroll
            for (int c = 0; c < K; ++c) tot[c] = hbuf[c] + (join ? sprev[c] : 0.0);
            if (head_before_unit) {
                a.head_row[u] = hrow;
                store_row<K>(a.head_val + (long long)u * K, tot);
            } else if (fits) {
                store_row<K>(rbuf + (hrow - RA) * KP, tot);
            } else {
                double *yr = y + out_row(M, hrow) * ldy;
#pragma unroll
                for (int c = 0; c < K; ++c) yr[c] = fin(tot[c], yr + c);
            }
        }
        const int last = cntu > 0 ? (cntu - 1) / S : 0;
        const bool unit_tail = lane == last && has_tail;
        if (unit_tail) {
            a.tail_row[u] = trow;
            store_row<K>(a.tail_val + (long long)u * K, sv);
        }
        const unsigned hb = __ballot_sync(FULL, head_before_unit);
        const unsigned tb = __ballot_sync(FULL, unit_tail);
        if (lane == 0) {
            if (hb == 0u) a.head_row[u] = -1;
            if (tb == 0u) a.tail_row[u] = -1;
        }
        __syncwarp();

        // ---- epilogue: the unit's complete rows, coalesced -----------------
        const int E0 = (rp(RA) < U0) ? RA + 1 : RA;
        if (fits) {
            const int ne = (RB - E0) * K;
            for (int i = lane; i < ne; i += 32) {
                const int rr = i / K, c = i - rr * K;
                double *yp = y + out_row(M, E0 + rr) * ldy + c;
                *yp = fin(rbuf[(E0 - RA + rr) * KP + c], yp);
            }
        } else {
            for (int r = E0 + lane; r < RB; r += 32)
                if (__ldg(rowptr + r) == __ldg(rowptr + r + 1)) {
                    double *yr = y + out_row(M, r) * ldy;
#pragma unroll
                    for (int c = 0; c < K; ++c) yr[c] = fin(0.0, yr + c);
                }
        }
    }
}

// ---- lanes over the right-hand sides (K >= 8) ------------------------------
// The same units, carries and fix-up as batch_spmm_kernel, another layout:
// a warp is 32 / K groups of K lanes, lane k of a group holds column k of
// the running row sum, and the group walks its own K * S consecutive
// nonzeros of the unit in order.  Per nonzero a group issues one K-wide
// coalesced load of the row of X and one FMA per lane, so a lane carries one
// accumulator instead of K: few registers, many warps per SM, and 32 DFMAs
// per warp instruction (the one-lane-per-chunk layout held 16 accumulators
// and 216 registers at K = 16).  The warp stages the unit's columns and
// values in shared memory first (coalesced; a group's entries at a stride of
// H + 1 so that the groups' broadcast reads fall in different banks), then
// every group takes its nonzeros in batches of VB, all loads of X of a
// batch issued before its first FMA.  Rows finished inside a group are
// written to Y at once (alpha, beta applied); each group's first row (begun
// before it) and last row (continuing past it) are joined in group order by
// the lanes of group 0, which write the rows completed inside the unit and
// the unit's head and tail carries for batch_fixup_kernel.  Empty rows of
// the unit are written by the whole warp at the end.
constexpr int VB = 8;    // nonzeros per batch of a group

template <int K, int S, int VK>
struct VecSmem {         // one warp
    static constexpr int G = 32 / K;
    static constexpr int H = K * S;
    static constexpr int SLOTS = 32 * S + G;     // group g's entries at g * (H + 1)
    static constexpr size_t COL = 0;
    static constexpr size_t VAL = (size_t(SLOTS) * 4 + 15) / 16 * 16;
    static constexpr size_t HV = (VAL + size_t(SLOTS) * VT<VK>::B + 15) / 16 * 16;
    static constexpr size_t TV = HV + size_t(G) * K * 8;
    static constexpr size_t ROWS = TV + size_t(G) * K * 8;   // hrow[G], trow[G], mid[G]
    static constexpr size_t TOTAL = (ROWS + size_t(3) * G * 4 + 15) / 16 * 16;
};

template <int K, int S, int VK>
constexpr size_t vec_cta_smem_bytes() { return size_t(NW) * VecSmem<K, S, VK>::TOTAL; }

template <int K, int S, int VK>
__global__ void __launch_bounds__(CTA, 8) batch_spmm_vec_kernel(const Args a)
{
    static_assert(K >= 4 && K <= 16 && (K & (K - 1)) == 0, "K in 4, 8, 16");
    using WS = VecSmem<K, S, VK>;
    constexpr int G = WS::G;
    constexpr int H = WS::H;
    static_assert(H % VB == 0, "whole batches per group");
    using T = typename VT<VK>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane / K, k = lane - g * K;
    unsigned char *ws = smem_raw + size_t(warp) * WS::TOTAL;
    int *scol = reinterpret_cast<int *>(ws + WS::COL);
    T *sval = reinterpret_cast<T *>(ws + WS::VAL);
    double *mhv = reinterpret_cast<double *>(ws + WS::HV);
    double *mtv = reinterpret_cast<double *>(ws + WS::TV);
    int *mhrow = reinterpret_cast<int *>(ws + WS::ROWS);
    int *mtrow = mhrow + G;
    int *mmid = mtrow + G;
    const uint64_t pol_x = ptx::policy_evict_last();

    for (int u = blockIdx.x * NW + warp; u < a.nunits; u += gridDim.x * NW) {
        const int b = __ldg(a.unit_mat + u);
        const Mat *M = a.mats + b;
        const int *rowptr = M->rowptr;
        const void *val = (a.override_xy && a.val) ? a.val : M->val;
        const double *x = a.override_xy ? a.x : M->x;
        double *y = a.override_xy ? a.y : M->y;
        const int ldx = a.override_xy ? a.ldx : M->ldx;
        const int ldy = a.override_xy ? a.ldy : M->ldy;
        const double alpha = a.override_xy ? a.alpha : M->alpha;
        const double beta = a.override_xy ? a.beta : M->beta;
        // alpha and beta classified once per unit: a finished row costs no
        // FP64 operation for alpha = 1, beta = 0 (the FP64 pipe bounds this
        // kernel, and a compare of doubles runs on it too)
        const int abmode = (beta != 0.0) ? 2 : (alpha != 1.0) ? 1 : 0;
        auto fin = [&](double v, double *yp) -> double {
            return abmode == 0 ? v : abmode == 1 ? alpha * v : fma(alpha, v, beta * *yp);
        };
        const int m = M->m;
        const int lu = u - M->unit0;
        const int U0 = lu * 32 * S;
        const int cntu = (int)min((long long)(32 * S), M->nnz - U0);
        const int RA = __ldg(a.unit_row + u);
        const int RB = (lu + 1 < M->nunits) ? __ldg(a.unit_row + u + 1) : m;

        // ---- stage the unit: columns and values (coalesced) -----------------
        __syncwarp();   // the previous unit's reads of the staging area are done
        for (int i = lane; i < cntu; i += 32) {
            const int slot = i + i / H;
            scol[slot] = __ldcs(M->col + U0 + i);
            if constexpr (VK != VAL_PATTERN) {
                const T *vp = static_cast<const T *>(val);
                sval[slot] = M->val_perm ? __ldg(vp + __ldcs(M->val_perm + U0 + i))
                                         : __ldcs(vp + U0 + i);
            }
        }
        __syncwarp();

        // ---- this group's nonzeros [gs, ge) ---------------------------------
        const int gs = U0 + min(g * H, cntu);
        const int ge = U0 + min((g + 1) * H, cntu);
        int r = RA, next = 0;
        bool sb = false, first = true;
        if (gs < ge) {
            int lo = RA, hi = min(RB, m - 1);   // last row starting at or before gs
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(rowptr + mid) <= gs) lo = mid; else hi = mid - 1;
            }
            r = lo;
            sb = __ldg(rowptr + r) < gs;
            next = __ldg(rowptr + r + 1);
        }
        const int s0 = g * (H + 1);          // slot of the group's first nonzero
        double acc = 0.0, head = 0.0;
        int hrow = -1;
        for (int b0 = gs; b0 < ge; b0 += VB) {
            const int nb = min(VB, ge - b0);
            const int sl = s0 + (b0 - gs);
            double xv[VB];
#pragma unroll
            for (int i = 0; i < VB; ++i)
                xv[i] = (i < nb) ? ptx::ldg_x_issue(x + (long long)scol[sl + i] * ldx + k, pol_x)
                                 : 0.0;
#pragma unroll
            for (int i = 0; i < VB; ++i) {
                if (i < nb) {
                    if (b0 + i == next) {
                        // row r ends before this nonzero
                        if (first && sb) {
                            head = acc;
                            hrow = r;
                        } else {
                            double *yp = y + out_row(M, r) * ldy + k;
                            *yp = fin(acc, yp);
                        }
                        first = false;
                        acc = 0.0;
                        ++r;
                        next = __ldg(rowptr + r + 1);
                        while (next == b0 + i) {   // empty rows: written at the unit's end
                            ++r;
                            next = __ldg(rowptr + r + 1);
                        }
                    }
                    if constexpr (VK == VAL_PATTERN) acc += xv[i];
                    else if constexpr (VK == VAL_F32) acc = fma(widen(sval[sl + i]), xv[i], acc);
                    else acc = fma(sval[sl + i], xv[i], acc);
                }
            }
        }
        // the group's last row: ends at the group's end, or continues past it
        int trow = -1;
        bool mid = false;
        if (gs < ge) {
            if (next == ge) {
                if (first && sb) {
                    head = acc;
                    hrow = r;
                } else {
                    double *yp = y + out_row(M, r) * ldy + k;
                    *yp = fin(acc, yp);
                }
            } else {
                trow = r;
                mid = first && sb;
            }
        }
        mhv[g * K + k] = head;
        mtv[g * K + k] = acc;
        if (k == 0) {
            mhrow[g] = hrow;
            mtrow[g] = trow;
            mmid[g] = mid ? 1 : 0;
        }
        __syncwarp();

        // ---- groups joined in order by group 0: rows crossing groups --------
        if (g == 0) {
            bool pend = false, uhead = false;
            int prow = -1;
            double pval = 0.0;
            for (int gg = 0; gg < G; ++gg) {
                const int hr = mhrow[gg];
                if (hr >= 0) {
                    const double h = mhv[gg * K + k];
                    const double tot = (pend && prow == hr) ? pval + h : h;
                    pend = false;
                    if (__ldg(rowptr + hr) < U0) {   // begun in an earlier unit: the head carry
                        a.head_val[(long long)u * K + k] = tot;
                        uhead = true;
                        if (k == 0) a.head_row[u] = hr;
                    } else {
                        double *yp = y + out_row(M, hr) * ldy + k;
                        *yp = fin(tot, yp);
                    }
                }
                const int tr = mtrow[gg];
                if (tr >= 0) {
                    const double t = mtv[gg * K + k];
                    pval = (mmid[gg] && pend && prow == tr) ? pval + t : t;
                    prow = tr;
                    pend = true;
                }
            }
            if (pend) a.tail_val[(long long)u * K + k] = pval;
            if (k == 0) {
                a.tail_row[u] = pend ? prow : -1;
                if (!uhead) a.head_row[u] = -1;
            }
        }
        // ---- empty rows of the unit ------------------------------------------
        const int E0 = (__ldg(rowptr + RA) < U0) ? RA + 1 : RA;
        for (int rr = E0 + lane; rr < RB; rr += 32)
            if (__ldg(rowptr + rr) == __ldg(rowptr + rr + 1)) {
                double *yr = y + out_row(M, rr) * ldy;
#pragma unroll
                for (int c = 0; c < K; ++c) yr[c] = fin(0.0, yr + c);
            }
    }
}

// ---- carry fix-up: rows crossing units ------------------------------------
// For every unit whose first row began in an earlier unit: that row's total
// is the unit's head plus the tails of the preceding units on the same row,
// added nearest first.
template <int K>
__global__ void batch_fixup_kernel(const Args a)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // whole warps iterate together (the cooperative path below needs them)
    for (int base = blockIdx.x * blockDim.x; base < a.nunits; base += gridDim.x * blockDim.x) {
        const int u = base + threadIdx.x;
        int R = (u < a.nunits) ? a.head_row[u] : -1;
        const Mat *M = (R >= 0) ? a.mats + __ldg(a.unit_mat + u) : nullptr;
        // a row spanning 32 or more earlier units (its units are contiguous,
        // so the unit 32 back carries the same row) is summed by the whole
        // warp; shorter runs by their own thread, nearest unit first
        const bool longrun = R >= 0 && u - 32 >= M->unit0 && a.tail_row[u - 32] == R;
        double t[K];
        if (R >= 0 && !longrun) {
#pragma unroll
            for (int c = 0; c < K; ++c) t[c] = a.head_val[(long long)u * K + c];
            for (int v = u - 1; v >= M->unit0 && a.tail_row[v] == R; --v) {
#pragma unroll
                for (int c = 0; c < K; ++c) t[c] += a.tail_val[(long long)v * K + c];
            }
        }
        unsigned pend = __ballot_sync(FULL, longrun);
        while (pend) {
            const int src = __ffs(pend) - 1;
            pend &= pend - 1;
            const int uu = __shfl_sync(FULL, u, src);
            const int RR = __shfl_sync(FULL, R, src);
            const int u0 = __shfl_sync(FULL, M ? M->unit0 : 0, src);
            // lane l sums units uu-1-l, uu-33-l, ... of the run
            double p[K];
#pragma unroll
            for (int c = 0; c < K; ++c) p[c] = 0.0;
            for (int top = uu - 1;; top -= 32) {
                const int v = top - lane;
                const bool in = v >= u0 && a.tail_row[v] == RR;
                if (in) {
#pragma unroll
                    for (int c = 0; c < K; ++c) p[c] += a.tail_val[(long long)v * K + c];
                }
                if (__ballot_sync(FULL, in) != FULL) break;
            }
            // fixed butterfly: the same order on every run
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
#pragma unroll
                for (int c = 0; c < K; ++c) p[c] += __shfl_xor_sync(FULL, p[c], d);
            }
            if (lane == src) {
#pragma unroll
                for (int c = 0; c < K; ++c) t[c] = a.head_val[(long long)u * K + c] + p[c];
            }
        }
        if (R >= 0) {
            double *y = a.override_xy ? a.y : M->y;
            const int ldy = a.override_xy ? a.ldy : M->ldy;
            const double alpha = a.override_xy ? a.alpha : M->alpha;
            const double beta = a.override_xy ? a.beta : M->beta;
            double *yr = y + out_row(M, R) * ldy;
#pragma unroll
            for (int c = 0; c < K; ++c) yr[c] = finish(t[c], alpha, beta, yr + c);
        }
    }
}

// ---- sampled dense-dense product over the pattern (values' adjoint) -------
// dval[p] = sum over c of G[row(p), c] * X[col(p), c] for every stored entry
// of a single-matrix plan; one warp per unit, lane l takes nonzeros
// U0 + l, U0 + l + 32, ... (coalesced col and dval), rows found by a binary
// search for the first and a forward walk after that.
template <int K, int S, int VK>
__global__ void __launch_bounds__(CTA) batch_sddmm_kernel(const Args a)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t pol = ptx::policy_evict_last();
    for (int u = blockIdx.x * NW + warp; u < a.nunits; u += gridDim.x * NW) {
        const Mat *M = a.mats + __ldg(a.unit_mat + u);
        const int *rowptr = M->rowptr;
        const int *col = M->col;
        const int lu = u - M->unit0;
        const int U0 = lu * 32 * S;
        const int cntu = (int)min((long long)(32 * S), M->nnz - U0);
        if (lane >= cntu) continue;
        const int RA = __ldg(a.unit_row + u);
        const int RB = (lu + 1 < M->nunits) ? __ldg(a.unit_row + u + 1) : M->m - 1;
        int p = U0 + lane;
        int lo = RA, hi = min(RB, M->m - 1);
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(rowptr + mid) <= p) lo = mid; else hi = mid - 1;
        }
        int r = lo;
        int next = __ldg(rowptr + r + 1);
        for (int i = lane; i < cntu; i += 32, p += 32) {
            while (next <= p) {
                ++r;
                next = __ldg(rowptr + r + 1);
            }
            double gr[K], xr[K];
            gather_row<K>(a.g, out_row(M, r), a.ldg, gr, pol);
            gather_row<K>(a.x, __ldcs(col + p), a.ldx, xr, pol);
            // four independent partial sums, joined at the end: the dependent
            // DFMA latency is long on this GPU (two partial sums, one join
            // less, measured slower: 0.70 -> 0.76 ms on the autograd matrix)
            constexpr int NP = K >= 4 ? 4 : K;
            double part[NP];
#pragma unroll
            for (int q = 0; q < NP; ++q) part[q] = 0.0;
#pragma unroll
            for (int c = 0; c < K; ++c) part[c % NP] = fma(gr[c], xr[c], part[c % NP]);
            double d;
            if constexpr (NP == 4) d = (part[0] + part[1]) + (part[2] + part[3]);
            else if constexpr (NP == 2) d = part[0] + part[1];
            else d = part[0];
            if constexpr (VK == VAL_F32) static_cast<float *>(a.dval)[p] = (float)d;
            else static_cast<double *>(a.dval)[p] = d;
        }
    }
}

// Launch of one compiled shape (main kernel + fix-up) on `stream`.
// K >= 8 runs the lanes-over-columns kernel, K <= 4 the lane-per-chunk
// kernel.  Measured on a 1M-row power-law matrix (20.1M nonzeros) and the
// 64-matrix batch: K = 16 0.76 ms against 1.14 ms (one lane per chunk, as
// two K = 8 passes), K = 8 batch 6.27 against 7.02 ms; K = 4 batch 4.22
// against 3.42 ms (at K = 4 a group's row of X is one sector and the
// one-lane-per-chunk layout keeps its FP64 pipe busier).
template <int K>
constexpr bool use_vec() { return K >= 8; }

template <int K, int S, int VK>
cudaError_t launch_shape(const Args &a, int grid, cudaStream_t stream)
{
    if (a.nunits <= 0) return cudaSuccess;
    if constexpr (use_vec<K>()) {
        batch_spmm_vec_kernel<K, S, VK><<<grid, CTA, vec_cta_smem_bytes<K, S, VK>(), stream>>>(a);
    } else {
        constexpr size_t smem = cta_smem_bytes<K, S, VK>();
        batch_spmm_kernel<K, S, VK><<<grid, CTA, smem, stream>>>(a);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int fgrid = (a.nunits + 255) / 256 < 1024 ? (a.nunits + 255) / 256 : 1024;
    batch_fixup_kernel<K><<<fgrid, 256, 0, stream>>>(a);
    return cudaGetLastError();
}

// Occupancy-sized persistent grid for one compiled shape (sets the dynamic
// shared-memory limit of the kernel first).
template <int K, int S, int VK>
cudaError_t shape_grid(int nunits, int *grid)
{
    size_t smem = 0;
    void (*kfn)(const Args);
    cudaError_t e = cudaSuccess;
    if constexpr (use_vec<K>()) {
        smem = vec_cta_smem_bytes<K, S, VK>();
        kfn = batch_spmm_vec_kernel<K, S, VK>;
    } else {
        smem = cta_smem_bytes<K, S, VK>();
        kfn = batch_spmm_kernel<K, S, VK>;
    }
    e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, bps = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn, CTA, smem)) != cudaSuccess)
        return e;
    if (bps < 1) return cudaErrorInvalidConfiguration;
    const long long need = (nunits + NW - 1) / NW;
    const long long full = (long long)sms * bps;
    *grid = (int)(need < full ? need : full);
    if (*grid < 1) *grid = 1;
    return cudaSuccess;
}

}  // namespace batch
}  // namespace sblas

namespace sblas {
namespace batch {

// Compiled shapes: K in {1, 2, 4, 8, 16} (one translation unit each),
// S in {4, 8, 16, 32}, every value kind.  Op::GRID computes the persistent
// grid of the shape into *grid_out; SPMM and SDDMM launch.
template <int K, int S, int VK>
cudaError_t launch_sddmm(const Args &a, int grid, cudaStream_t stream)
{
    if constexpr (VK == VAL_PATTERN) {
        return cudaErrorInvalidValue;
    } else {
        if (a.nunits <= 0) return cudaSuccess;
        batch_sddmm_kernel<K, S, VK><<<grid, CTA, 0, stream>>>(a);
        return cudaGetLastError();
    }
}

enum class Op { GRID, SPMM, SDDMM };

template <int K>
cudaError_t dispatch_k(Op op, int S, int VK, const Args *a, int nunits, int grid, int *grid_out,
                       cudaStream_t stream)
{
#define SBLAS_BATCH_SHAPE(SS, VV)                                                        \
    if (S == SS && VK == VV)                                                             \
        return op == Op::SPMM    ? launch_shape<K, SS, VV>(*a, grid, stream)             \
               : op == Op::SDDMM ? launch_sddmm<K, SS, VV>(*a, grid, stream)             \
                                 : shape_grid<K, SS, VV>(nunits, grid_out);
#define SBLAS_BATCH_S(SS)                                                                \
    SBLAS_BATCH_SHAPE(SS, VAL_F64) SBLAS_BATCH_SHAPE(SS, VAL_F32) SBLAS_BATCH_SHAPE(SS, VAL_PATTERN)
    SBLAS_BATCH_S(4)
    SBLAS_BATCH_S(8)
    SBLAS_BATCH_S(16)
    SBLAS_BATCH_S(32)
#undef SBLAS_BATCH_S
#undef SBLAS_BATCH_SHAPE
    return cudaErrorInvalidValue;
}

}  // namespace batch
}  // namespace sblas
