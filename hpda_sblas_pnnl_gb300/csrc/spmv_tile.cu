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
// Design for GB300 (measured: the FP64 pipe retires ~1.65e10 warp
// instructions/s whatever the number of active lanes, i.e. ~0.53 T DFMA/s;
// random 32-byte L2->SM gathers run at ~2.8e11/s, one per nonzero):
//  * warp-specialised persistent CTA: 4 compute warps (one chunk of SIGMA
//    nonzeros per lane), a producer warp staging tiles into a STAGES-deep
//    shared-memory ring with 1-D bulk copies (cp.async.bulk, L2 evict-first),
//    and two epilogue warps (one per tile parity) merging the chunk carries
//    one tile behind;
//    mbarrier hand-offs, every wait bounded, no CTA-wide barrier in the loop;
//  * each lane finds its chunk's rows in the staged row-pointer slice
//    (binary search + row-start bits) before it issues the chunk's gathers:
//    issued after them, the search's dependent shared-memory reads waited
//    behind the gathers in the load pipeline;
//  * every lane runs exactly SIGMA fused multiply-adds with all 32 lanes
//    active; a row ending inside the chunk only costs integer work and a
//    shared-memory store (the running sum restarts with a select);
//  * the per-lane partial of the row crossing a chunk boundary ("tail") is
//    combined by an epilogue warp: runs of equal rows reduced lane-
//    sequentially (NCW adds per lane, work-efficient) and a 5-step segmented
//    shuffle scan joining runs crossing lanes; the lane that holds the end of
//    the row adds the result to its partial ("head") once;
//  * rows are finished in a coalesced epilogue (alpha/beta applied once per
//    row, nothing at all when alpha = 1 and beta = 0);
//  * the row crossing a tile boundary is finished by a tiny fix-up kernel
//    that adds the FP64 carries in a fixed order (no atomics: results are
//    bit-reproducible run to run);
//  * x is gathered with an L2 evict-last hint; grids are persistent
//    (occupancy x SM count), tiles round-robin over CTAs.
#include <atomic>
#include <cstdio>
#include <climits>
#include <mutex>

#include <utility>

#include "ptx.cuh"
#include "sblas_internal.h"

namespace sblas {

namespace {

constexpr int STAGES = 2;
constexpr uint64_t DEFAULT_WAIT_NS = 2000000000ull;  // 2 s per wait, then error flag

// Device error codes written to status[0].
constexpr int DEV_ERR_TIMEOUT = 1;

// Sticky per-device error word: every launch whose bounded wait gave up ORs
// its code in, whatever workspace it ran with; read (and cleared) by
// sblas_stream_status for the asynchronous entry points.
__device__ int g_sticky_error;

// Wait limit of the compute and epilogue warps and of the producer's wait
// for a free stage (the producer's final wait for its own copies always
// uses DEFAULT_WAIT_NS), and the test hook that holds the producer back.
std::atomic<unsigned long long> g_wait_ns{DEFAULT_WAIT_NS};
std::atomic<int> g_stall{0};

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

constexpr int NCW = 4;                 // compute warps per CTA
constexpr int TC = NCW * 32;           // compute threads per CTA (one chunk each)
constexpr int NEW = 2;                 // epilogue warps: one per tile parity
constexpr int CTA_THREADS = TC + 32 + 32 * NEW;   // + producer warp + epilogue warps

// Shared-memory bytes of one CTA (the Layout below) for a row capacity r.
template <int SIGMA, int VK>
constexpr size_t layout_bytes(int r)
{
    const size_t tile = size_t(TC) * SIGMA;
    const size_t rslot = size_t((r + 8 + 3) / 4 * 4);
    const size_t col = align16(size_t(STAGES) * tile * ValTraits<VK>::BYTES);
    const size_t rptr = align16(col + size_t(STAGES) * tile * 4);
    const size_t meta = align16(rptr + size_t(STAGES) * rslot * 4);
    const size_t rval = align16(meta + size_t(STAGES) * 16);
    const size_t tailv = align16(rval + 2 * size_t(r) * 8);
    const size_t cmeta = align16(tailv + 4 * size_t(TC) * 8 + 4 * size_t(TC) * 4);
    return align16(cmeta + 2 * 16) + (2 * STAGES + 4) * 8;
}

// Rows of a tile held in shared memory: TILE / 4 + 2, unless the CTAs that
// fit on an SM (at most 5: 54-62 registers x 224 threads at sigma = 11, fewer
// for the larger shapes) would then need more than 196 KB of shared memory
// per SM.  Past that the driver takes the 228-KB carveout, leaves about
// 28 KB of L1, and random gathers of x run at less than half their rate; the
// row capacity is then trimmed (by a quarter at most) until the same CTA
// count fits in 196 KB.  Shapes that still do not fit get a padded request
// at launch (configure_shape).
template <int SIGMA, int VK>
constexpr int rows_in_smem()
{
    constexpr size_t kLimit = size_t(195) * 1024;   // 196 KB less a 1-KB margin
    const int r = TC * SIGMA / 4 + 2;
    const size_t cta = layout_bytes<SIGMA, VK>(r) + 1024;   // + the driver's 1 KB per CTA
    int occ = (int)(size_t(228 * 1024) / cta);
    if (occ > 5) occ = 5;
    if ((size_t)occ * cta <= kLimit) return r;
    const size_t budget = kLimit / occ - 1024;
    int t = r;
    while (t > r - r / 4 && layout_bytes<SIGMA, VK>(t) > budget) --t;
    return layout_bytes<SIGMA, VK>(t) <= budget ? t : r;
}

template <int SIGMA, int VK>
struct Layout {
    static constexpr int TILE = TC * SIGMA;
    static constexpr int RCAP = rows_in_smem<SIGMA, VK>();  // owned rows (+2) of a tile held
                                                            // in smem; denser tiles use the
                                                            // global-memory path
    static constexpr int RSLOT = (RCAP + 8 + 3) / 4 * 4;  // per-stage row-pointer slot
    static constexpr int VB = ValTraits<VK>::BYTES;
    // staged tiles
    static constexpr size_t VAL = 0;
    static constexpr size_t COL = align16(VAL + size_t(STAGES) * TILE * VB);
    static constexpr size_t RPTR = align16(COL + size_t(STAGES) * TILE * 4);
    static constexpr size_t META = align16(RPTR + size_t(STAGES) * RSLOT * 4);
    // carry buffers, double-buffered by tile parity
    static constexpr size_t RVAL = align16(META + size_t(STAGES) * 16);
    static constexpr size_t TAILV = align16(RVAL + 2 * size_t(RCAP) * 8);
    static constexpr size_t HEADV = TAILV + 2 * size_t(TC) * 8;
    static constexpr size_t TAILK = HEADV + 2 * size_t(TC) * 8;
    static constexpr size_t HEADK = TAILK + 2 * size_t(TC) * 4;
    static constexpr size_t CMETA = align16(HEADK + 2 * size_t(TC) * 4);
    // mbarriers: full[STAGES], empty[STAGES], cfull[2], cempty[2]
    static constexpr size_t BAR = align16(CMETA + 2 * 16);
    static constexpr size_t TOTAL = BAR + (2 * STAGES + 4) * 8;
};

static_assert(layout_bytes<19, VAL_F64>(Layout<19, VAL_F64>::RCAP) == Layout<19, VAL_F64>::TOTAL,
              "layout_bytes follows Layout");
static_assert(layout_bytes<15, VAL_F32>(Layout<15, VAL_F32>::RCAP) == Layout<15, VAL_F32>::TOTAL,
              "layout_bytes follows Layout");
static_assert(layout_bytes<27, VAL_PATTERN>(Layout<27, VAL_PATTERN>::RCAP) ==
                  Layout<27, VAL_PATTERN>::TOTAL,
              "layout_bytes follows Layout");

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
    int stall;            // test hook: the producer stages nothing, every wait runs out
    uint64_t wait_ns;     // limit of one bounded wait
};

// What a tile needs of the matrix it belongs to.
struct MatView {
    int m;
    long long nnz;
    long long tb;          // first nonzero of the tile, inside its matrix
    const void *val;
    const int *rowptr;
    const int *col;
    const double *x;
    double *y;
    double alpha;
    double beta;
    int use_tma;
    int rp_tma;
    const int *part;       // part[0], part[1]: the rows the tile owns, [R0, R1)
    double *carry;         // the tile's carry slot
    int abmode;            // runtime alpha/beta (AB = 3): 0 alpha = 1, beta = 0;
                           // 1 beta = 0; 2 general (classified on the host)
};

// Source of tiles: one matrix (TileArgs) or many (MultiArgs, below).  Both
// give the total tile count, a tile's matrix and the tile's view of it.
__device__ __forceinline__ int mat_of(const TileArgs &, int) { return 0; }

template <int TILE>
__device__ __forceinline__ MatView view_of(const TileArgs &a, int tile, int)
{
    return MatView{a.m,      a.nnz,   (long long)tile * TILE, a.val,   a.rowptr,
                   a.col,    a.x,     a.y,                    a.alpha, a.beta,
                   a.use_tma, a.rp_tma, a.row_part + tile,    a.carry + tile, 2};
}

// One matrix of a multi-matrix launch (the batched single-right-hand-side
// form): its tiles are global tiles [tile0, tile0 + ntiles), its partition
// part[part_off .. part_off + ntiles].
struct MultiMat {
    const void *val;
    const int *rowptr;
    const int *col;
    const double *x;
    double *y;
    long long nnz;
    int m;
    int tile0;
    int part_off;
    int use_tma;
    int rp_tma;
    double alpha;
    double beta;
    int abmode;   // 0: alpha = 1, beta = 0; 1: beta = 0; 2: general
};

struct MultiArgs {
    const MultiMat *mats;
    const int *tile0s;    // [nmat + 1]: first global tile of every matrix, then the total
    int nmat;
    int ntiles;
    const int *part;
    double *carry;        // [ntiles], by global tile
    int *status;
    int stall;
    uint64_t wait_ns;
};

__device__ __forceinline__ int mat_of(const MultiArgs &a, int tile)
{
    int lo = 0, hi = a.nmat - 1;   // last matrix with tile0 <= tile
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(a.tile0s + mid) <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <int TILE>
__device__ __forceinline__ MatView view_of(const MultiArgs &a, int tile, int mat)
{
    const MultiMat *M = a.mats + mat;
    const int lt = tile - M->tile0;
    return MatView{M->m,       M->nnz,    (long long)lt * TILE, M->val,  M->rowptr,
                   M->col,     M->x,      M->y,                 M->alpha, M->beta,
                   M->use_tma, M->rp_tma, a.part + M->part_off + lt, a.carry + tile,
                   M->abmode};
}

// A bounded wait gave up: the launch's status word and the sticky word.
template <class Src>
__device__ __forceinline__ void report_timeout(const Src &a)
{
    atomicExch(a.status, DEV_ERR_TIMEOUT);
    atomicOr(&g_sticky_error, DEV_ERR_TIMEOUT);
}

// y epilogue for one finished row value v.  AB = 3: alpha and beta known
// only at run time (matrices of a multi-matrix launch each have their own).
template <int AB>
__device__ __forceinline__ double finish_row(double v, double alpha, double beta,
                                             const double *yp, int abmode)
{
    if (AB == 0) return v;                               // alpha = 1, beta = 0
    if (AB == 1) return alpha * v;                       // beta = 0
    // AB = 3: the matrix's case, classified on the host (a compare of
    // doubles per row would run on the FP64 pipe)
    if (AB == 3 && abmode != 2) return abmode == 0 ? v : alpha * v;
    return fma(alpha, v, beta * __ldg(yp));              // general
}

template <int SIGMA, int VK>
struct Smem {
    using L = Layout<SIGMA, VK>;
    using VT = typename ValTraits<VK>::T;
    unsigned char *base;
    __device__ VT *val(int s) const { return reinterpret_cast<VT *>(base + L::VAL) + size_t(s) * L::TILE; }
    __device__ int *col(int s) const { return reinterpret_cast<int *>(base + L::COL) + size_t(s) * L::TILE; }
    __device__ int *rptr(int s) const { return reinterpret_cast<int *>(base + L::RPTR) + size_t(s) * L::RSLOT; }
    __device__ int *meta(int s) const { return reinterpret_cast<int *>(base + L::META) + 4 * s; }
    __device__ double *rval(int p) const { return reinterpret_cast<double *>(base + L::RVAL) + size_t(p) * L::RCAP; }
    __device__ double *tailv(int p) const { return reinterpret_cast<double *>(base + L::TAILV) + p * TC; }
    __device__ double *headv(int p) const { return reinterpret_cast<double *>(base + L::HEADV) + p * TC; }
    __device__ int *tailk(int p) const { return reinterpret_cast<int *>(base + L::TAILK) + p * TC; }
    __device__ int *headk(int p) const { return reinterpret_cast<int *>(base + L::HEADK) + p * TC; }
    __device__ int *cmeta(int p) const { return reinterpret_cast<int *>(base + L::CMETA) + 4 * p; }
    __device__ uint64_t *bar() const { return reinterpret_cast<uint64_t *>(base + L::BAR); }
    __device__ uint64_t *full(int s) const { return bar() + s; }
    __device__ uint64_t *empty(int s) const { return bar() + STAGES + s; }
    __device__ uint64_t *cfull(int p) const { return bar() + 2 * STAGES + p; }
    __device__ uint64_t *cempty(int p) const { return bar() + 2 * STAGES + 2 + p; }
};

// Stages tile `tile` into stage `s` (the producer warp, all lanes): owned-row
// range (R0, R1), val and col by bulk copy, the row-pointer slice
// rowptr[R0 .. R1+1] by bulk copy of its 16-byte-aligned superset; ragged
// ends (and everything when a pointer is not 16-byte aligned) by plain loads
// of the 32 lanes.  Completion: the stage's `full` mbarrier (one arrive with
// the byte count, after the plain stores).
template <int SIGMA, int VK>
__device__ __forceinline__ void produce_tile(const MatView &a, const Smem<SIGMA, VK> &sm,
                                             int mat, int s, int R0, int R1, int lane,
                                             uint64_t pol)
{
    using L = Layout<SIGMA, VK>;
    using VT = typename ValTraits<VK>::T;
    const long long tb = a.tb;
    const int cnt = (int)((a.nnz - tb < L::TILE) ? (a.nnz - tb) : L::TILE);
    const int vdone = a.use_tma ? (int)((((long long)cnt * L::VB) & ~15ll) / (L::VB ? L::VB : 1)) : 0;
    const int cdone = a.use_tma ? (int)((((long long)cnt * 4) & ~15ll) / 4) : 0;
    const int nr = R1 - R0;
    const int fits = (nr + 2) <= L::RCAP;
    int base = R0, t_end = R0, a1 = R0;
    if (fits) {
        const int count = min(nr + 2, a.m - R0 + 1);   // rowptr[R0 .. R0+count-1]
        a1 = R0 + count;
        if (a.rp_tma) {
            base = R0 & ~3;
            const int safe_end = (a.m + 1) & ~3;        // bulk copies stay inside rowptr
            t_end = max(base, min((a1 + 3) & ~3, safe_end));
        }
    }
    VT *vst = sm.val(s);
    int *cst = sm.col(s);
    int *rslot = sm.rptr(s);
    if (VK != VAL_PATTERN)
        for (int i = vdone + lane; i < cnt; i += 32) vst[i] = static_cast<const VT *>(a.val)[tb + i];
    for (int i = cdone + lane; i < cnt; i += 32) cst[i] = __ldg(a.col + tb + i);
    for (int i = t_end + lane; i < a1; i += 32) rslot[i - base] = __ldg(a.rowptr + i);
    if (lane == 0) {
        int *meta = sm.meta(s);
        meta[0] = R0;
        meta[1] = R1;
        meta[2] = base;
        meta[3] = fits | (mat << 1);   // the tile's matrix rides with the flag
    }
    __syncwarp();
    if (lane == 0) {
        const uint32_t vbytes = (uint32_t)vdone * L::VB;
        const uint32_t cbytes = (uint32_t)cdone * 4u;
        const uint32_t rbytes = (uint32_t)(t_end - base) * 4u;
        ptx::mbar_arrive_expect_tx(sm.full(s), vbytes + cbytes + rbytes);  // release
        if (vbytes)
            ptx::bulk_g2s(vst, static_cast<const unsigned char *>(a.val) + tb * L::VB, vbytes,
                          sm.full(s), pol);
        if (cbytes) ptx::bulk_g2s(cst, a.col + tb, cbytes, sm.full(s), pol);
        if (rbytes) ptx::bulk_g2s(rslot, a.rowptr + base, rbytes, sm.full(s), pol);
    }
}

// FP32 value widened to FP64 exactly with integer operations: sign, the
// exponent rebased by 1023 - 127 (2047 for infinities and NaNs), the 23-bit
// significand moved to the top of the 52-bit field; a subnormal is first
// scaled by 2^64 in FP32 (exact) and its exponent lowered by 64 again.  F2F
// conversions run on the FP64 pipe of this GPU, which the multiply-adds
// already keep busy; these run on the integer and FP32 pipes.
__device__ __forceinline__ double widen_f32(float v)
{
    const unsigned u0 = __float_as_uint(v);
    const bool sub = (u0 & 0x7F800000u) == 0u && (u0 << 1) != 0u;
    const unsigned u = sub ? __float_as_uint(v * 0x1p64f) : u0;
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned ed = (e == 0xFFu) ? 0x7FFu : (e == 0u ? 0u : e + 896u - (sub ? 64u : 0u));
    const unsigned hi = (u & 0x80000000u) | (ed << 20) | ((u >> 3) & 0xFFFFFu);
    return __hiloint2double((int)hi, (int)(u << 29));
}

// The same widening for a normal FP32 number (exponent field 1..254): sign,
// exponent rebased by 896 and significand moved in three integer
// operations.  The compute warps take it for a chunk when no lane's chunk
// holds a zero, a subnormal, an infinity or a NaN (their exponent field is 0
// or 255: ((bits >> 23) + 1) & 0xFE == 0), which a warp vote decides; the
// general widening above costs about twice the instructions, and on the
// banded matrix the FP32 form was bound by instruction issue.
__device__ __forceinline__ double widen_normal_f32(unsigned u)
{
    const unsigned hi = (((u & 0x7FFFFFFFu) >> 3) + 0x38000000u) | (u & 0x80000000u);
    return __hiloint2double((int)hi, (int)(u << 29));
}

__device__ __forceinline__ bool f32_not_normal(unsigned u)
{
    return (((u >> 23) + 1u) & 0xFEu) == 0u;
}

// Compute warp: for each tile of the CTA, one chunk of SIGMA consecutive
// nonzeros per lane.  Row sums completed inside the chunk go to the carry
// buffer of the tile's parity; the chunk's head (first segment of a row
// begun earlier) and tail (partial of the row crossing the chunk end) are
// published for the epilogue warp of the tile's parity.  No CTA-wide barrier.
template <int SIGMA, int VK, int AB, class Src>
__device__ __forceinline__ void compute_warp(const Src &src, const Smem<SIGMA, VK> &sm,
                                             int cw, int lane, uint64_t pol_x)
{
    using L = Layout<SIGMA, VK>;
    using VT = typename ValTraits<VK>::T;
    constexpr int TILE = L::TILE;
    const int t = cw * 32 + lane;
    for (int i = 0, tile = blockIdx.x; tile < src.ntiles; ++i, tile += gridDim.x) {
        const int s = i % STAGES;
        const int p = i & 1;
        bool ok = ptx::mbar_wait_bounded(sm.full(s), (uint32_t)((i / STAGES) & 1), src.wait_ns);
        if (i >= 2)
            ok = ok && ptx::mbar_wait_bounded(sm.cempty(p), (uint32_t)(((i - 2) / 2) & 1),
                                              src.wait_ns);
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) report_timeout(src);
            return;
        }
        const int *meta = sm.meta(s);
        const int R0 = meta[0], R1 = meta[1], rbase = meta[2];
        const bool fits = (meta[3] & 1) != 0;
        const int mat = meta[3] >> 1;
        const MatView a = view_of<TILE>(src, tile, mat);
        const double alpha = a.alpha, beta = a.beta;
        const long long tb = a.tb;
        const int cnt_tile = (int)((a.nnz - tb < TILE) ? (a.nnz - tb) : TILE);
        const VT *vst = sm.val(s);
        const int *cst = sm.col(s);
        const int *rptr_s = sm.rptr(s);
        double *rval = sm.rval(p);

        const int c0 = t * SIGMA;                            // local offset in tile
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
            // the chunk's rows first: the dependent shared-memory reads of
            // the search would otherwise wait behind the gathers in the
            // load pipeline.  Last row r in [R0, R1] with rowptr[r] <= s0
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
            // then every gather of the chunk (one L2 round trip per chunk
            // instead of one per nonzero)
            if (cnt == SIGMA) {
#pragma unroll
                for (int j = 0; j < SIGMA; ++j)
                    xv[j] = ptx::ldg_x_issue(a.x + cst[c0 + j], pol_x);
            } else {
#pragma unroll
                for (int j = 0; j < SIGMA; ++j)
                    xv[j] = ptx::ldg_x_issue(a.x + cst[c0 + (j < cnt ? j : 0)], pol_x);
            }
        }
        const bool warp_slow = __any_sync(0xffffffffu, slow);
        double sum = 0.0;
        bool f32_odd = false;   // FP32: this lane's chunk holds a value that is not normal
        int head_row = -1;
        double head_val = 0.0;
        double *headv = sm.headv(p);
        // branch-free FMA chain: at a row start the running sum is stored
        // (the first segment to the thread's head slot when the row began in
        // an earlier chunk) and restarted with a select
        auto chain = [&](auto value_of) {
            sum = 0.0;
            double *dst = sb ? &headv[t] : &rval[r0 - R0];
            double *nxt = &rval[r0 + 1 - R0];
#pragma unroll
            for (int j = 0; j < SIGMA; ++j) {
                const bool b = (mask >> j) & 1u;
                if (b) *dst = sum;
                dst = b ? nxt : dst;
                nxt = b ? nxt + 1 : nxt;
                sum = b ? 0.0 : sum;
                if (j < cnt) {
                    if constexpr (VK == VAL_PATTERN) sum += xv[j];
                    else sum = fma(value_of(j), xv[j], sum);
                }
            }
        };
        if (cnt > 0 && !warp_slow) {
            if constexpr (VK == VAL_F32) {
                // FP32 values read once: the chain widens them the short way
                // (exact for normal numbers) and notes any zero, subnormal,
                // infinity or NaN; a warp holding one redoes its chains with
                // the general widening below, which rewrites the same row
                // slots (a second read of every value in the common case was
                // as much shared-memory traffic as FP64 values)
                unsigned odd = 0u;
                chain([&](int j) {
                    const unsigned u = __float_as_uint(vst[c0 + j]);
                    odd |= f32_not_normal(u) ? 1u : 0u;
                    return widen_normal_f32(u);
                });
                f32_odd = odd != 0u;
            } else {
                chain([&](int j) { return (double)vst[c0 + j]; });
            }
            if (sb && mask != 0u) head_row = r0;
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
                        rval[r - R0] = sum;
                    } else {
                        a.y[r] = finish_row<AB>(sum, alpha, beta, a.y + r, a.abmode);
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
            headv[t] = head_val;
        }
        if constexpr (VK == VAL_F32) {
            // every lane votes (also lanes without data or on the general path)
            if (__any_sync(0xffffffffu, f32_odd) && cnt > 0 && !warp_slow)
                chain([&](int j) { return widen_f32(vst[c0 + j]); });
        }
        // tails stored transposed (thread t at (t % NCW) * 32 + t / NCW) so that
        // the carry pass, where lane l reads threads l*NCW .. l*NCW+NCW-1, is
        // free of shared-memory bank conflicts
        const int tslot = (t % NCW) * 32 + t / NCW;
        sm.tailv(p)[tslot] = sum;
        sm.tailk(p)[tslot] = (cnt > 0) ? rl : -1;   // -1: no data, never emitted
        sm.headk(p)[t] = head_row;
        if (t == 0) {
            int *cm = sm.cmeta(p);
            cm[0] = R0;
            cm[1] = R1;
            cm[2] = fits;
            cm[3] = mat;
        }
        __syncwarp();
        if (lane == 0) {
            ptx::mbar_arrive(sm.empty(s));   // stage s may be refilled
            ptx::mbar_arrive(sm.cfull(p));   // carry buffers of this tile published
        }
    }
}

// Producer warp: stages the CTA's tiles into the STAGES-deep ring, each as
// soon as the compute warps release its stage; the tile's partition entries
// are loaded before that wait, so their latency hides behind it.
template <int SIGMA, int VK, class Src>
__device__ __forceinline__ void producer_warp(const Src &src, const Smem<SIGMA, VK> &sm,
                                              int lane, uint64_t pol_stream)
{
    constexpr int TILE = Layout<SIGMA, VK>::TILE;
    if (src.stall) return;   // test hook: nothing is staged, the other warps' waits run out
    int issued[STAGES];
#pragma unroll
    for (int s = 0; s < STAGES; ++s) issued[s] = 0;
    for (int s = 0; s < STAGES; ++s) {
        const int t = blockIdx.x + s * (int)gridDim.x;
        if (t < src.ntiles) {
            const int mat = mat_of(src, t);
            const MatView v = view_of<TILE>(src, t, mat);
            produce_tile<SIGMA, VK>(v, sm, mat, s, __ldg(v.part), __ldg(v.part + 1), lane,
                                    pol_stream);
            ++issued[s];
        }
    }
    for (int i = 0, nt = blockIdx.x + STAGES * (int)gridDim.x; nt < src.ntiles;
         ++i, nt += gridDim.x) {
        const int s = i % STAGES;
        const int mat = mat_of(src, nt);
        const MatView v = view_of<TILE>(src, nt, mat);
        const int R0 = __ldg(v.part);
        const int R1 = __ldg(v.part + 1);
        const bool ok = ptx::mbar_wait_bounded(sm.empty(s), (uint32_t)((i / STAGES) & 1),
                                               src.wait_ns);
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) report_timeout(src);
            break;
        }
        ptx::fence_proxy_async_smem();
        produce_tile<SIGMA, VK>(v, sm, mat, s, R0, R1, lane, pol_stream);
        ++issued[s];
    }
    // the CTA may exit only when no copy into its shared memory is in flight
    // (always the full limit: these copies are this warp's own and complete)
    if (lane == 0) {
        for (int s = 0; s < STAGES; ++s)
            if (issued[s] > 0)
                ptx::mbar_wait_bounded(sm.full(s), (uint32_t)((issued[s] - 1) & 1),
                                       DEFAULT_WAIT_NS);
    }
}

// Epilogue warp: one tile behind the compute warps, merges the chunk
// carries of each tile and writes its rows.
//   carry pass: runs of equal rows among the TC tails are reduced lane-
//   sequentially (NCW tails per lane, work-efficient), a 5-step segmented
//   shuffle scan joins runs crossing lanes; each run total goes to the head
//   of the chunk where the row ends, to a complete row, or to the tile carry;
//   head pass: the heads (with the run each joins, added by the carry pass:
//   an add only where a run meets a head) out to their rows;
//   epilogue: alpha/beta once per row, coalesced stores of y.
template <int SIGMA, int VK, int AB, class Src>
__device__ __forceinline__ void epilogue_warp(const Src &src, const Smem<SIGMA, VK> &sm,
                                              int par, int lane)
{
    constexpr int PER = NCW;  // tails reduced per lane
    constexpr int TILE = Layout<SIGMA, VK>::TILE;
    // this warp takes the tiles of parity `par` (the CTA's tiles i = par,
    // par + 2, ...): the carry buffers are double-buffered by that parity
    for (int i = par, tile = blockIdx.x + par * (int)gridDim.x; tile < src.ntiles;
         i += 2, tile += 2 * (int)gridDim.x) {
        const int p = i & 1;
        const bool ok = ptx::mbar_wait_bounded(sm.cfull(p), (uint32_t)((i / 2) & 1),
                                               src.wait_ns);
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) report_timeout(src);
            break;
        }
        const int *cm = sm.cmeta(p);
        const int R0 = cm[0], R1 = cm[1];
        const bool fits = cm[2] != 0;
        const MatView a = view_of<TILE>(src, tile, cm[3]);
        const double alpha = a.alpha, beta = a.beta;
        double *rval = sm.rval(p);
        const double *tailv = sm.tailv(p);
        const int *tailk = sm.tailk(p);
        const int *headk = sm.headk(p);
        double *headv = sm.headv(p);

        // ---------------- carry pass -------------------------------------
        {
            auto emit = [&](int key, double total, int after) {
                if (key < 0) return;
                if (after < TC && headk[after] == key) {
                    headv[after] += total;                   // joins a head (its one run)
                } else if (after >= TC && key == R1) {
                    *a.carry = total;                        // continues in next tile
                } else if (fits) {
                    rval[key - R0] = total;                  // complete row
                } else {
                    a.y[key] = finish_row<AB>(total, alpha, beta, a.y + key, a.abmode);
                }
            };
            if (lane == 0) *a.carry = 0.0;
            __syncwarp();
            const int base = lane * PER;          // first thread of this lane's tails
            double acc = 0.0;
            int prevk = tailk[lane];              // thread base at slot 0*32 + lane
            const int fk = prevk;
            double af = 0.0;
            int f_after = base + PER;
            bool broke = false;
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int ii = base + q;          // thread index (heads use it)
                const int key = tailk[q * 32 + lane];
                const bool brk = (q > 0) && (key != prevk);
                if (brk) {
                    if (!broke) {
                        af = acc;
                        f_after = ii;
                        broke = true;
                    } else {
                        emit(prevk, acc, ii);
                    }
                }
                // the first tail starts the sum (no add: partial sums are
                // never -0, so 0 + t == t bit for bit); the FP64 pipe bounds
                // the banded matrices, and every add here is one of its slots
                if (q == 0) acc = tailv[lane];
                else acc = (brk ? 0.0 : acc) + tailv[q * 32 + lane];
                prevk = key;
            }
            const bool single = !broke;
            const int kl = prevk;
            double S = acc;
            const int kl_prev = __shfl_up_sync(0xffffffffu, kl, 1);
            bool f = (lane == 0) || !single || (kl != kl_prev);
            // segmented scan across lanes, only where a lane's last run
            // continues from its left neighbour somewhere in the warp, and
            // only as many steps as the longest such chain of lanes needs
            // (the steps after those add 0 to every lane)
            const unsigned contm = __ballot_sync(0xffffffffu, !f);
            if (contm != 0u) {
                const unsigned starts = ~contm & ((2u << lane) - 1u);
                const int lrun = lane - (31 - __clz(starts));   // lanes joined from the left
                const int maxrun = (int)__reduce_max_sync(0xffffffffu, (unsigned)lrun);
                for (int d = 1; d <= maxrun; d <<= 1) {
                    const double So = __shfl_up_sync(0xffffffffu, S, d);
                    const bool fo = __shfl_up_sync(0xffffffffu, f, d);
                    const bool take = (lane >= d) && !f;
                    S = S + (take ? So : 0.0);
                    f = take ? fo : f;
                }
            }
            const double S_prev = __shfl_up_sync(0xffffffffu, S, 1);
            // first run of a lane with several runs may continue from the left
            const double tot = af + ((lane > 0 && kl_prev == fk) ? S_prev : 0.0);
            if (!single) emit(fk, tot, f_after);
            // last run ends here unless the next lane starts with the same row
            const int next_first = (lane < 31) ? tailk[lane + 1] : INT_MIN;
            if (lane == 31 || next_first != kl) emit(kl, S, base + PER);
        }
        __syncwarp();
        // ---------------- head pass: heads out to their rows ---------------
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int tt = q * 32 + lane;
            const int hr = headk[tt];
            const double hv = headv[tt];   // the head with the run it joins added
            if (hr >= 0) {
                if (fits) rval[hr - R0] = hv;
                else a.y[hr] = finish_row<AB>(hv, alpha, beta, a.y + hr, a.abmode);
            }
        }
        __syncwarp();
        // ---------------- epilogue: finished rows out, slots cleared ------
        const int nr = R1 - R0;
        if (fits) {
            for (int r = lane; r < nr; r += 32) {
                a.y[R0 + r] = finish_row<AB>(rval[r], alpha, beta, a.y + R0 + r, a.abmode);
                rval[r] = 0.0;
            }
        } else {
            for (int rr = R0 + lane; rr < R1; rr += 32)
                if (__ldg(a.rowptr + rr) == __ldg(a.rowptr + rr + 1))
                    a.y[rr] = finish_row<AB>(0.0, alpha, beta, a.y + rr, a.abmode);
        }
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(sm.cempty(p));
    }
}

// CTAs per SM the registers must allow: five for the sigma = 11 shapes
// whose shared memory fits five (FP32 values, pattern-only), else no bound.
template <int SIGMA, int VK>
constexpr int min_ctas() { return (SIGMA == 11 && VK != VAL_F64) ? 5 : 1; }

template <int SIGMA, int VK, int AB, class Src>
__global__ void __launch_bounds__(CTA_THREADS, min_ctas<SIGMA, VK>()) tile_spmv_kernel(const Src a)
{
    using L = Layout<SIGMA, VK>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const Smem<SIGMA, VK> sm{smem_raw};
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            ptx::mbar_init(sm.full(s), 1);
            ptx::mbar_init(sm.empty(s), NCW);
        }
        for (int p = 0; p < 2; ++p) {
            ptx::mbar_init(sm.cfull(p), NCW);
            ptx::mbar_init(sm.cempty(p), 1);
        }
        ptx::fence_mbar_init();
    }
    for (int i = tid; i < 2 * L::RCAP; i += CTA_THREADS) sm.rval(0)[i] = 0.0;
    __syncthreads();
    // launched right behind the tile partition: the set-up above overlapped
    // its end; nothing in global memory is read before it has finished
    ptx::griddep_wait();
    if (warp == NCW)
        producer_warp<SIGMA, VK, Src>(a, sm, lane, ptx::policy_evict_first());
    else if (warp > NCW)
        epilogue_warp<SIGMA, VK, AB, Src>(a, sm, warp - NCW - 1, lane);
    else
        compute_warp<SIGMA, VK, AB, Src>(a, sm, warp, lane, ptx::policy_evict_last());
}

// part[k] = number of rows r with rowptr[r+1] <= k*TILE (k = 1..ntiles-1);
// part[0] = 0, part[ntiles] = m.  Row r is owned by the tile holding its
// last nonzero; empty rows by the tile holding the nonzero before them.
// One streaming pass over the row pointer: the row r with
// rowptr[r] <= k*TILE < rowptr[r+1] is the only one whose count is r, so
// every non-empty row writes its own value into the entries it covers.
// Tiles k (1 <= k < ntiles) whose first nonzero k*tile lies in row r =
// [b, e) get part[k] = r.  One 32-bit division per row (64-bit divisions,
// two per row, made this pass issue-bound): most rows hold no tile start,
// and the second division only runs for rows that do.
__device__ __forceinline__ void own_tiles(int r, int b, int e, int ntiles, unsigned tile,
                                          int *__restrict__ part)
{
    if (e <= b) return;
    const unsigned k1 = (unsigned)(e - 1) / tile;             // last k with k*tile <= e-1
    const unsigned long long top = (unsigned long long)k1 * tile;
    if (top < (unsigned long long)b) return;                   // no tile starts in the row
    unsigned k = k1 - (unsigned)((top - (unsigned long long)b) / tile);   // first k*tile >= b
    if (k < 1u) k = 1u;
    for (; k <= k1 && k < (unsigned)ntiles; ++k) part[k] = r;
}

__global__ void tile_partition_kernel(int m, long long nnz, int ntiles, long long tile,
                                      const int *__restrict__ rowptr, int *__restrict__ part)
{
    (void)nnz;
    ptx::griddep_launch_dependents();   // the tile kernel may start its set-up
    const int stride = gridDim.x * blockDim.x;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g == 0) {
        part[0] = 0;
        part[ntiles] = m;
    }
    for (int r = g; r < m; r += stride)
        own_tiles(r, __ldg(rowptr + r), __ldg(rowptr + r + 1), ntiles, (unsigned)tile, part);
}

// The same pass for a 16-byte aligned row pointer: four rows per thread from
// one 16-byte load (plus the next entry), two such loads in flight; one row
// per thread kept too few bytes in flight to stream the row pointer.
__global__ void tile_partition_quad_kernel(int m, int ntiles, long long tile,
                                           const int *__restrict__ rowptr,
                                           int *__restrict__ part)
{
    ptx::griddep_launch_dependents();   // the tile kernel may start its set-up
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g == 0) {
        part[0] = 0;
        part[ntiles] = m;
    }
    const long long nq = m / 4;
    const int4 *q4 = reinterpret_cast<const int4 *>(rowptr);
    const unsigned t32 = (unsigned)tile;
    auto quad = [&](const int4 v, int next, long long r0) {
        own_tiles((int)r0, v.x, v.y, ntiles, t32, part);
        own_tiles((int)r0 + 1, v.y, v.z, ntiles, t32, part);
        own_tiles((int)r0 + 2, v.z, v.w, ntiles, t32, part);
        own_tiles((int)r0 + 3, v.w, next, ntiles, t32, part);
    };
    for (long long q = g; q < nq; q += 2 * stride) {
        const long long q2 = q + stride;
        const bool two = q2 < nq;
        const int4 v = __ldg(q4 + q);
        const int ve = __ldg(rowptr + 4 * q + 4);
        const int4 w = two ? __ldg(q4 + q2) : v;
        const int we = two ? __ldg(rowptr + 4 * q2 + 4) : 0;
        quad(v, ve, 4 * q);
        if (two) quad(w, we, 4 * q2);
    }
    for (long long r = 4 * nq + g; r < m; r += stride)
        own_tiles((int)r, __ldg(rowptr + r), __ldg(rowptr + r + 1), ntiles, t32, part);
}

// Adds the carries of the tiles a row spans to the row, in tile order.
__global__ void tile_fixup_kernel(int ntiles, long long tile, double alpha,
                                  const int *__restrict__ rowptr, const int *__restrict__ part,
                                  const double *__restrict__ carry, double *__restrict__ y,
                                  const int *__restrict__ status)
{
    ptx::griddep_wait();   // launched behind the tile kernel: its carries are complete
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

// tile_fixup_kernel for a multi-matrix launch: global tile k, its matrix's
// own tiles and partition.
__global__ void multi_fixup_kernel(const MultiArgs a, long long tile)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.ntiles) return;
    if (*a.status != 0) return;
    const MultiMat *M = a.mats + mat_of(a, k);
    const int lt = k - M->tile0;
    if (lt == 0) return;                                        // a matrix's first tile
    const int *part = a.part + M->part_off;
    const int r = part[lt];
    if (part[lt + 1] <= r) return;                              // row r ends later
    if ((long long)__ldg(M->rowptr + r) >= (long long)lt * tile) return;   // starts here
    int j = lt - 1;
    double c = a.carry[M->tile0 + j];
    while (j >= 1 && part[j] == part[j + 1]) {
        c += a.carry[M->tile0 + j - 1];
        --j;
    }
    M->y[r] = fma(M->alpha, c, M->y[r]);
}

// ---------------- compiled shapes -----------------------------------------
constexpr int kSigmas[] = {11, 15, 19, 23, 27};
constexpr int kNumSigmas = sizeof(kSigmas) / sizeof(kSigmas[0]);

// Per device: the kernel's shared-memory attribute, set once, its resident
// CTAs per SM (0 = not configured yet) and the dynamic shared memory each
// launch requests; host threads may launch concurrently.  Configuring also
// loads the kernel onto the device under lazy module loading.
//
// Random gathers of x run at less than half their rate once the CTAs of an
// SM hold more than 196 KB of shared memory (the driver then takes the
// largest carveout and leaves ~28 KB of L1).  rows_in_smem trims each
// shape's row buffer for four CTAs per SM; a shape whose registers let a
// fifth CTA in (the smaller layouts: FP32 values and pattern-only at
// sigma = 11, ~54 registers) would pass the limit again, so the request is
// padded until the CTAs that fit stay within it (one CTA fewer), down to two
// CTAs per SM.
template <int SIGMA, int VK, int AB, class Src = TileArgs>
int configure_shape(int *out_bps, size_t *out_smem)
{
    using L = Layout<SIGMA, VK>;
    auto kfn = tile_spmv_kernel<SIGMA, VK, AB, Src>;
    constexpr int kMaxDev = 64;
    constexpr size_t kSmemLimit = size_t(195) * 1024;   // per SM, with the 1 KB per CTA
    static std::atomic<int> blocks_per_sm[kMaxDev];
    static size_t smem_request[kMaxDev];
    static std::mutex config_mu;
    int dev = 0;
    SBLAS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDev) {
        set_error(SBLAS_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
        return SBLAS_ERR_UNSUPPORTED;
    }
    int bps = blocks_per_sm[dev].load(std::memory_order_acquire);
    if (bps == 0) {
        std::lock_guard<std::mutex> lk(config_mu);
        bps = blocks_per_sm[dev].load(std::memory_order_acquire);
        if (bps == 0) {
            size_t req = L::TOTAL;
            for (;;) {
                SBLAS_CUDA_TRY(cudaFuncSetAttribute(
                    kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)req));
                SBLAS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn,
                                                                             CTA_THREADS, req));
                // (never down to one CTA per SM: measured slower than the
                // small-L1 carveout with two, banded sigma 27 947 -> 1464 us)
                if (bps <= 2 || (size_t)bps * (req + 1024) <= kSmemLimit) break;
                // just enough that one CTA fewer fits in the SM's 228 KB
                const size_t next = ((size_t(228) * 1024 / bps - 1024 + 128) + 127) & ~size_t(127);
                if (next <= req || next > size_t(227) * 1024) break;
                req = next;
            }
            if (bps < 1) {
                set_error(SBLAS_ERR_UNSUPPORTED, "tile shape sigma=%d does not fit on this GPU",
                          SIGMA);
                return SBLAS_ERR_UNSUPPORTED;
            }
            smem_request[dev] = req;
            blocks_per_sm[dev].store(bps, std::memory_order_release);
        }
    }
    *out_bps = bps;
    if (out_smem) *out_smem = smem_request[dev];
    return SBLAS_OK;
}

// A launch with programmatic stream serialisation: the kernel may start
// while the previous kernel of the stream finishes, and waits for it
// (ptx::griddep_wait) before it reads global memory.
template <class... KArgs, class... Args>
cudaError_t launch_pdl(void (*kfn)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t stream, Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kfn, std::forward<Args>(args)...);
}

template <int SIGMA, int VK, int AB, class Src = TileArgs>
int launch_shape(const Src &a, cudaStream_t stream)
{
    auto kfn = tile_spmv_kernel<SIGMA, VK, AB, Src>;
    int bps = 0;
    size_t smem = 0;
    const int rc = configure_shape<SIGMA, VK, AB, Src>(&bps, &smem);
    if (rc != SBLAS_OK) return rc;
    const int grid = min(a.ntiles, bps * device_num_sms());
    SBLAS_CUDA_TRY(launch_pdl(kfn, dim3(grid), dim3(CTA_THREADS), smem, stream, a));
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
TileShape tile_shape_at(int i) { return TileShape{TC, kSigmas[i]}; }
int tile_shape_index(int sigma)
{
    for (int i = 0; i < kNumSigmas; ++i)
        if (kSigmas[i] == sigma) return i;
    return -1;
}

static size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// Workspace layout: the status word (first 256 bytes, at the same place
// whatever the matrix, so launches of different sizes on one workspace share
// it), then the tile partition, then the tile carries.
constexpr size_t kStatusBytes = 256;

size_t tile_workspace_bytes(long long nnz, int sigma)
{
    const long long tile = (long long)TC * sigma;
    const long long ntiles = (nnz + tile - 1) / tile;
    return kStatusBytes + align256(sizeof(int) * (size_t)(ntiles + 1)) +
           align256(sizeof(double) * (size_t)ntiles);
}

int default_sigma_for(int m, long long nnz)
{
    // measured best on both benchmark matrices (power-law 312 us, banded
    // 802 us; sigma 15: 317 / 830, 19: 327 / 935); the tuner measures the
    // caller's own matrix
    (void)m;
    (void)nnz;
    return 11;
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
    const long long tile = (long long)TC * sigma;
    const long long ntiles_ll = (nnz + tile - 1) / tile;
    if (ntiles_ll > INT_MAX - 2) {
        set_error(SBLAS_ERR_ARG, "nnz %lld too large", nnz);
        return SBLAS_ERR_ARG;
    }
    const int ntiles = (int)ntiles_ll;
    int *part = reinterpret_cast<int *>(static_cast<unsigned char *>(work) + kStatusBytes);
    const int threads = 256;
    if ((reinterpret_cast<uintptr_t>(rowptr) & 15) == 0) {
        const int quads = m / 4 + 1;
        const int blocks = min((quads + threads - 1) / threads, 8 * device_num_sms());
        tile_partition_quad_kernel<<<blocks, threads, 0, stream>>>(m, ntiles, tile, rowptr,
                                                                   part);
    } else {
        const int blocks = min((m + threads - 1) / threads, 8 * device_num_sms());
        tile_partition_kernel<<<blocks, threads, 0, stream>>>(m, nnz, ntiles, tile, rowptr,
                                                              part);
    }
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

// Status word of a tile workspace (after the partition and the carries).
static int *status_in(void *work) { return static_cast<int *>(work); }

int tile_workspace_status(void *work, int *out)
{
    *out = 0;
    if (work == nullptr) return SBLAS_OK;
    SBLAS_CUDA_TRY(cudaMemcpy(out, status_in(work), sizeof(int), cudaMemcpyDeviceToHost));
    return SBLAS_OK;
}

int tile_sticky_status(cudaStream_t stream, bool clear, int *out)
{
    *out = 0;
    SBLAS_CUDA_TRY(cudaMemcpyFromSymbolAsync(out, g_sticky_error, sizeof(int), 0,
                                             cudaMemcpyDeviceToHost, stream));
    SBLAS_CUDA_TRY(cudaStreamSynchronize(stream));
    if (clear && *out != 0) {
        const int zero = 0;
        SBLAS_CUDA_TRY(cudaMemcpyToSymbolAsync(g_sticky_error, &zero, sizeof(int), 0,
                                               cudaMemcpyHostToDevice, stream));
        SBLAS_CUDA_TRY(cudaStreamSynchronize(stream));
    }
    return SBLAS_OK;
}

// Configures (and so loads) every kernel an FP64 SpMV of tile shape sigma
// may launch on the current device.
int tile_preload_f64(int sigma)
{
    int bps = 0, rc = SBLAS_OK;
    switch (sigma) {
#define SBLAS_PRELOAD(S)                                                            \
    case S:                                                                         \
        rc = configure_shape<S, VAL_F64, 0>(&bps, nullptr);                         \
        if (rc == SBLAS_OK) rc = configure_shape<S, VAL_F64, 1>(&bps, nullptr);     \
        if (rc == SBLAS_OK) rc = configure_shape<S, VAL_F64, 2>(&bps, nullptr);     \
        break;
        SBLAS_PRELOAD(11)
        SBLAS_PRELOAD(15)
        SBLAS_PRELOAD(19)
        SBLAS_PRELOAD(23)
        SBLAS_PRELOAD(27)
#undef SBLAS_PRELOAD
    default:
        set_error(SBLAS_ERR_UNSUPPORTED, "sigma %d is not a compiled tile shape", sigma);
        return SBLAS_ERR_UNSUPPORTED;
    }
    if (rc != SBLAS_OK) return rc;
    cudaFuncAttributes fa;
    SBLAS_CUDA_TRY(cudaFuncGetAttributes(&fa, tile_partition_kernel));
    SBLAS_CUDA_TRY(cudaFuncGetAttributes(&fa, tile_partition_quad_kernel));
    SBLAS_CUDA_TRY(cudaFuncGetAttributes(&fa, tile_fixup_kernel));
    SBLAS_CUDA_TRY(cudaFuncGetAttributes(&fa, scale_y_kernel));
    return SBLAS_OK;
}

int multi_tile_sigma() { return 11; }

size_t multi_tile_count(long long nnz)
{
    const long long tile = (long long)TC * multi_tile_sigma();
    return nnz <= 0 ? 1 : (size_t)((nnz + tile - 1) / tile);
}

int launch_tile_partition(int m, long long nnz, const int *rowptr, int sigma, int *part,
                          cudaStream_t stream)
{
    // launch_tile_analyse writes the partition after the status word
    return launch_tile_analyse(m, nnz, rowptr, sigma,
                               reinterpret_cast<unsigned char *>(part) - kStatusBytes, stream);
}

int launch_multi_tile_spmv(const MultiTileLaunch &L, int val_kind, cudaStream_t stream)
{
    if (L.ntiles <= 0) return SBLAS_OK;
    MultiArgs a;
    a.mats = static_cast<const MultiMat *>(L.mats);
    a.tile0s = L.tile0s;
    a.nmat = L.nmat;
    a.ntiles = L.ntiles;
    a.part = L.part;
    a.carry = L.carry;
    a.status = L.status;
    a.stall = g_stall.load(std::memory_order_relaxed);
    a.wait_ns = g_wait_ns.load(std::memory_order_relaxed);
    SBLAS_CUDA_TRY(cudaMemsetAsync(L.status, 0, sizeof(int), stream));
    int rc;
    switch (val_kind) {
    case VAL_F64: rc = launch_shape<11, VAL_F64, 3, MultiArgs>(a, stream); break;
    case VAL_F32: rc = launch_shape<11, VAL_F32, 3, MultiArgs>(a, stream); break;
    case VAL_PATTERN: rc = launch_shape<11, VAL_PATTERN, 3, MultiArgs>(a, stream); break;
    default:
        set_error(SBLAS_ERR_ARG, "unknown value kind %d", val_kind);
        return SBLAS_ERR_ARG;
    }
    if (rc != SBLAS_OK) return rc;
    if (a.ntiles > 1) {
        const int threads = 256;
        multi_fixup_kernel<<<(a.ntiles + threads - 1) / threads, threads, 0, stream>>>(
            a, (long long)TC * multi_tile_sigma());
        SBLAS_CUDA_TRY(cudaGetLastError());
    }
    return SBLAS_OK;
}

size_t multi_mat_bytes() { return sizeof(MultiMat); }

void fill_multi_mat(void *dst, const void *val, const int *rowptr, const int *col,
                    const double *x, double *y, long long nnz, int m, int tile0, int part_off,
                    double alpha, double beta, int val_kind)
{
    MultiMat M;
    M.val = val;
    M.rowptr = rowptr;
    M.col = col;
    M.x = x;
    M.y = y;
    M.nnz = nnz;
    M.m = m;
    M.tile0 = tile0;
    M.part_off = part_off;
    const uintptr_t vb = reinterpret_cast<uintptr_t>(val), cb = reinterpret_cast<uintptr_t>(col);
    M.use_tma = ((val_kind == VAL_PATTERN || (vb & 15) == 0) && (cb & 15) == 0) ? 1 : 0;
    M.rp_tma = (reinterpret_cast<uintptr_t>(rowptr) & 15) == 0 ? 1 : 0;
    M.alpha = alpha;
    M.beta = beta;
    M.abmode = (beta != 0.0) ? 2 : (alpha != 1.0) ? 1 : 0;
    *static_cast<MultiMat *>(dst) = M;
}

void set_wait_limit_ns(unsigned long long ns)
{
    g_wait_ns.store(ns == 0 ? DEFAULT_WAIT_NS : ns, std::memory_order_relaxed);
}

void set_test_stall(int on) { g_stall.store(on ? 1 : 0, std::memory_order_relaxed); }

int launch_tile_spmv(int m, int n, long long nnz, double alpha, const void *val, int val_kind,
                     const int *rowptr, const int *col, const double *x, double beta, double *y,
                     int sigma, void *work, cudaStream_t stream, bool analysed, bool reset_status)
{
    if (m <= 0) return SBLAS_OK;
    if (nnz <= 0) return launch_scale_y(m, beta, y, stream);
    if (tile_shape_index(sigma) < 0) {
        set_error(SBLAS_ERR_UNSUPPORTED, "sigma %d is not a compiled tile shape", sigma);
        return SBLAS_ERR_UNSUPPORTED;
    }
    const long long tile = (long long)TC * sigma;
    const long long ntiles_ll = (nnz + tile - 1) / tile;
    if (ntiles_ll > INT_MAX - 2) {
        set_error(SBLAS_ERR_ARG, "nnz %lld too large", nnz);
        return SBLAS_ERR_ARG;
    }
    const int ntiles = (int)ntiles_ll;
    unsigned char *w = static_cast<unsigned char *>(work);
    int *part = reinterpret_cast<int *>(w + kStatusBytes);
    double *carry = reinterpret_cast<double *>(w + kStatusBytes +
                                               align256(sizeof(int) * (size_t)(ntiles + 1)));
    int *status = status_in(work);
    if (reset_status) SBLAS_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), stream));
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
    a.stall = g_stall.load(std::memory_order_relaxed);
    a.wait_ns = g_wait_ns.load(std::memory_order_relaxed);
    int rc = SBLAS_OK;
    switch (sigma) {
    case 11: rc = launch_vk<11>(val_kind, a, stream); break;
    case 15: rc = launch_vk<15>(val_kind, a, stream); break;
    case 19: rc = launch_vk<19>(val_kind, a, stream); break;
    case 23: rc = launch_vk<23>(val_kind, a, stream); break;
    case 27: rc = launch_vk<27>(val_kind, a, stream); break;
    default: rc = SBLAS_ERR_UNSUPPORTED; break;
    }
    if (rc != SBLAS_OK) return rc;
    if (ntiles > 1) {
        const int threads = 256;
        const int blocks = (ntiles - 1 + threads - 1) / threads;
        SBLAS_CUDA_TRY(launch_pdl(tile_fixup_kernel, dim3(blocks), dim3(threads), 0, stream,
                                  ntiles, tile, alpha, rowptr, part, carry, y, status));
        SBLAS_CUDA_TRY(cudaGetLastError());
    }
    return SBLAS_OK;
}

}  // namespace sblas
