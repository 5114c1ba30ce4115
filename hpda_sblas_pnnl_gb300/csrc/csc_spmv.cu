// y = alpha*A*x + beta*y with A in CSC: atomic-free and deterministic.
//
// The reference runs its CSC entry points as a transposed cuSPARSE csrmv
// (src/dspmv_mgpu_baseline_csc.cu:131-135), 4-33x slower than its CSR path.
// Here the work is split into an inspector, once per sparsity pattern, and
// an executor, once per product:
//   inspector  the row-ordered structure of A: a stable least-significant-
//              digit bucket sort of the CSC entries by row (bucket_sort.cuh)
//              carrying each entry's column and CSC position, giving A's CSR
//              row pointer, columns and the permutation perm (CSR position ->
//              CSC position), then the tile partition of that row pointer;
//   executor   the values in row order, then the CSR tile kernel: its
//              segmented sums and carry fix-up in a fixed order, no atomics,
//              bit-reproducible.
// Two ways to put the values into row order:
//   direct     out[p] = val[perm[p]]: one random read of every value from
//              DRAM (the values do not fit in L2), used by the one-shot
//              product, whose inspector runs on every call;
//   staged     for an analysed pattern reused many times (sblas_csc_analyse):
//              the row-order positions are cut into buckets of 2^bits
//              (8 MB of values).  The inspector adds two index arrays:
//              dst[q], the slot of CSC entry q in a staging array that holds
//              every bucket's values contiguously (in CSC order inside the
//              bucket), and src[p], the staging slot of row position p, inside
//              p's own bucket.  The executor streams the values once into the
//              staging array (sequential reads; each tile regrouped by bucket
//              in shared memory, so the writes are runs) and then gathers
//              each bucket from its 8 MB window, which stays in L2: two
//              streaming passes instead of a random DRAM read per value.
// sblas_dcscmv runs inspector and executor; sblas_csc_analyse /
// sblas_dcscmv_analysed split them, and sblas_csc_bind_values keeps one set
// of values in row order inside the analysis, so that products with those
// values cost a CSR product alone.
#include <algorithm>

#include "bucket_sort.cuh"
#include "sblas_internal.h"

namespace sblas {
namespace {

size_t al256(size_t v) { return (v + 255) & ~size_t(255); }

constexpr int kCscSigma = 11;     // tile shape of the executor (the library default)
constexpr int kStageBits = 20;    // staging bucket: 2^20 row positions (8 MB of values)

// Staging buckets of a matrix: nb is a power of two (the digit mask of the
// bucket pass), used = the buckets that hold entries; used == 1: no staging.
struct StagePlan {
    int bits, nb, used;
};

StagePlan stage_plan(long long nnz)
{
    StagePlan s{kStageBits, 1, 1};
    if (nnz <= 1) return s;
    while (((nnz - 1) >> s.bits) >= bsort::MAXB) ++s.bits;
    s.used = (int)(((nnz - 1) >> s.bits) + 1);
    while (s.nb < s.used) s.nb <<= 1;
    return s;
}

// Workspace: rowptr | col | perm (src when staged) | dst | runs | val (row
// order) | tile workspace | scratch (the inspector's sort, then its staging
// temporaries; the executor's staging array).  runs (staged only): for
// every staging tile t and bucket b < used, the first staging slot of the
// tile's entries in b (int, run_first[t * used + b]) and their count
// (unsigned short, after all the firsts).
struct CscLayout {
    size_t rowptr, col, perm, dst, runs, val, tile, scratch, total;
};

long long stage_tiles(long long nnz) { return bsort::num_tiles(nnz); }

CscLayout csc_layout(int m, int n, long long nnz)
{
    const size_t nn = (size_t)(nnz > 0 ? nnz : 1);
    const StagePlan sp = stage_plan(nnz);
    const bool staged = sp.used > 1;
    const size_t nruns = staged ? (size_t)stage_tiles(nnz) * (size_t)sp.used : 0;
    CscLayout L;
    L.rowptr = 0;
    L.col = L.rowptr + al256(4 * ((size_t)m + 1));
    L.perm = L.col + al256(4 * nn);
    L.dst = L.perm + al256(4 * nn);
    L.runs = L.dst + (staged ? al256(4 * nn) : 0);
    L.val = L.runs + (staged ? al256(4 * nruns) + al256(2 * nruns) : 0);
    L.tile = L.val + al256(8 * nn);
    L.scratch = L.tile + al256(tile_workspace_bytes(nnz, kCscSigma));
    size_t scratch = al256(csr_transpose_workspace_bytes(n, m, nnz));
    if (staged) {
        const size_t inspect = 2 * al256(4 * nn) + al256(bsort::pass_work_bytes(nnz, sp.nb));
        scratch = std::max(scratch, std::max(inspect, al256(8 * nn)));
    }
    L.total = L.scratch + scratch;
    return L;
}

// Index and value moves over nnz entries: one CTA per chunk of MOVE_CHUNK
// consecutive entries (CTAs start in index order, so the chunks in flight
// stay close together: the staged gather's reads fall in one or two
// L2-resident buckets), every thread MOVE_ILP entries 256 apart, all loads
// in flight before the first store.
constexpr int MOVE_THREADS = 256;
constexpr int MOVE_ILP = 8;
constexpr int MOVE_CHUNK = MOVE_THREADS * MOVE_ILP;

unsigned move_grid(long long nnz) { return (unsigned)((nnz + MOVE_CHUNK - 1) / MOVE_CHUNK); }

// out[p] = in[idx[p]]
__global__ void __launch_bounds__(MOVE_THREADS) gather_values_kernel(long long nnz,
                                                                    const int *__restrict__ idx,
                                                                    const double *__restrict__ in,
                                                                    double *__restrict__ out)
{
    const long long base = (long long)blockIdx.x * MOVE_CHUNK + threadIdx.x;
    int p[MOVE_ILP];
    double v[MOVE_ILP];
#pragma unroll
    for (int k = 0; k < MOVE_ILP; ++k) {
        const long long e = base + k * MOVE_THREADS;
        p[k] = e < nnz ? __ldg(idx + e) : -1;
    }
#pragma unroll
    for (int k = 0; k < MOVE_ILP; ++k)   // an index outside [0, nnz) reads nothing
        v[k] = (p[k] >= 0 && (long long)p[k] < nnz) ? __ldcg(in + p[k]) : 0.0;
#pragma unroll
    for (int k = 0; k < MOVE_ILP; ++k)
        if (base + k * MOVE_THREADS < nnz) out[base + k * MOVE_THREADS] = v[k];
}

// The staging scatter, stage[dst[q]] = val[q], one CTA per tile of
// bsort::TILE CSC entries: the tiles of the staging pass that made dst, so
// the tile's entries of one bucket hold consecutive slots, from the run's
// first slot on (runs, kept by the inspector).  The tile is regrouped in
// shared memory by bucket (slot = the run's offset in the tile + dst - the
// run's first slot), then every warp stores whole runs: consecutive lanes,
// consecutive slots.  No atomics: the run table gives every offset.
constexpr int STAGE_TILE = bsort::TILE;
static_assert(STAGE_TILE == MOVE_CHUNK, "staging tiles are the staging pass's tiles");

__global__ void __launch_bounds__(MOVE_THREADS) stage_scatter_kernel(
    long long nnz, int bits, int used, const int *__restrict__ dst,
    const int *__restrict__ run_first, const unsigned short *__restrict__ run_count,
    const double *__restrict__ in, double *__restrict__ out)
{
    __shared__ double st_val[STAGE_TILE];
    __shared__ int first[bsort::MAXB], cnt[bsort::MAXB], off[bsort::MAXB];
    __shared__ int wsum[MOVE_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const long long base = (long long)blockIdx.x * STAGE_TILE;
    const int len = (int)min((long long)STAGE_TILE, nnz - base);
    int d[MOVE_ILP];
    double v[MOVE_ILP];
#pragma unroll
    for (int k = 0; k < MOVE_ILP; ++k) {
        const int i = k * MOVE_THREADS + tid;
        d[k] = i < len ? __ldg(dst + base + i) : -1;
        v[k] = i < len ? __ldg(in + base + i) : 0.0;
    }
    const long long r0 = (long long)blockIdx.x * used;
    const int own = tid < used ? (int)__ldg(run_count + r0 + tid) : 0;
    if (tid < used) {
        first[tid] = __ldg(run_first + r0 + tid);
        cnt[tid] = own;
    }
    // exclusive scan of the run lengths (used <= 256: one per thread)
    int incl = own;
#pragma unroll
    for (int k = 1; k < 32; k <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, incl, k);
        if (lane >= k) incl += o;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    int before = 0;
#pragma unroll
    for (int k = 0; k < MOVE_THREADS / 32; ++k) before += k < w ? wsum[k] : 0;
    if (tid < used) off[tid] = before + incl - own;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < MOVE_ILP; ++k) {
        // a slot outside the run table (a workspace that no staged analysis
        // wrote) is dropped, never stored
        if (d[k] < 0 || (long long)d[k] >= nnz) continue;
        const int b = d[k] >> bits;
        if (b >= used) continue;
        const int r = d[k] - first[b];
        if (r >= 0 && r < cnt[b]) st_val[off[b] + r] = v[k];
    }
    __syncthreads();
    for (int b = w; b < used; b += MOVE_THREADS / 32) {
        const int f = first[b], c = cnt[b], o = off[b];
        if (f < 0 || (long long)f + c > nnz || o + c > STAGE_TILE) continue;
        for (int i = lane; i < c; i += 32) out[f + i] = st_val[o + i];
    }
}

// Run table of the staging tiles from the staging pass's scanned digit-major
// table (pos[b * ntiles + t] = first slot of tile t's entries in bucket b).
__global__ void stage_runs_kernel(long long nnz, int ntiles, int used, int nb,
                                  const int *__restrict__ pos, int *__restrict__ run_first,
                                  unsigned short *__restrict__ run_count)
{
    const long long total = (long long)ntiles * used;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long t = i / used, b = i - t * used;
        const long long flat = b * ntiles + t;
        const long long next = flat + 1 < (long long)nb * ntiles ? __ldg(pos + flat + 1) : nnz;
        const int f = __ldg(pos + flat);
        run_first[i] = f;
        run_count[i] = (unsigned short)(next - f);
    }
}

// out[idx[e]] = e: the inverse of a permutation (chunks as above, every
// index load in flight before the stores)
__global__ void __launch_bounds__(MOVE_THREADS) invert_kernel(long long nnz,
                                                             const int *__restrict__ idx,
                                                             int *__restrict__ out)
{
    const long long base = (long long)blockIdx.x * MOVE_CHUNK + threadIdx.x;
    int t[MOVE_ILP];
#pragma unroll
    for (int k = 0; k < MOVE_ILP; ++k) {
        const long long e = base + k * MOVE_THREADS;
        t[k] = e < nnz ? __ldg(idx + e) : -1;
    }
#pragma unroll
    for (int k = 0; k < MOVE_ILP; ++k)
        if (t[k] >= 0 && (long long)t[k] < nnz) out[t[k]] = (int)(base + k * MOVE_THREADS);
}

// The staging pass: CSC entries q keyed by their row position inv[q], one
// bucket digit (bits and up); the pass writes each entry's staging slot by
// CSC position (dst) and the row position held by every slot (key_out).
struct StageOp {
    const int *key_in;
    int *key_out;
    int *a_out = nullptr;
    int *b_out = nullptr;
    double *d_out = nullptr;
    int *pos_out;
    static constexpr bool kPosOut = true;
    struct State {};
    __device__ int key(long long e) const { return __ldg(key_in + e); }
    __device__ bsort::Payload load(State &, long long, int, bool, long long e) const
    {
        return bsort::Payload{0, (int)e, 0.0};
    }
};

bool check_work(int m, int n, long long nnz, void *work, size_t work_bytes)
{
    const size_t need = csc_layout(m, n, nnz).total;
    if (work == nullptr || work_bytes < need || (reinterpret_cast<uintptr_t>(work) & 255) != 0) {
        set_error(SBLAS_ERR_ARG, "CSC SpMV workspace needs %zu bytes at 256-byte alignment",
                  need);
        return false;
    }
    return true;
}

}  // namespace

size_t cscmv_workspace_bytes(int m, int n, long long nnz) { return csc_layout(m, n, nnz).total; }

int launch_csc_analyse(int m, int n, long long nnz, const int *colptr, const int *rowidx,
                       void *work, size_t work_bytes, bool staged, cudaStream_t stream)
{
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d n=%d nnz=%lld", m, n, nnz);
        return SBLAS_ERR_ARG;
    }
    if (m == 0 || nnz == 0) return SBLAS_OK;
    if (!check_work(m, n, nnz, work, work_bytes)) return SBLAS_ERR_ARG;
    const CscLayout L = csc_layout(m, n, nnz);
    unsigned char *w = static_cast<unsigned char *>(work);
    int *rowptr = reinterpret_cast<int *>(w + L.rowptr);
    int *perm = reinterpret_cast<int *>(w + L.perm);
    // the CSC arrays are the CSR arrays of A^T (n rows): its transpose is A
    // in CSR, with every entry's CSC position as the permutation
    int rc = launch_csr_transpose(n, m, nnz, colptr, rowidx, rowptr,
                                  reinterpret_cast<int *>(w + L.col), perm, w + L.scratch,
                                  L.total - L.scratch, stream);
    if (rc != SBLAS_OK) return rc;
    rc = launch_tile_analyse(m, nnz, rowptr, kCscSigma, w + L.tile, stream);
    if (rc != SBLAS_OK) return rc;
    const StagePlan sp = stage_plan(nnz);
    if (!staged || sp.used <= 1) return SBLAS_OK;
    // staging indices: inv (row position of CSC entry q), the bucket pass
    // giving dst and the row position of every slot, then src (the slot of
    // every row position) in place of perm
    const size_t nn = (size_t)nnz;
    int *inv = reinterpret_cast<int *>(w + L.scratch);
    int *slot_row = reinterpret_cast<int *>(w + L.scratch + al256(4 * nn));
    void *pass_work = w + L.scratch + 2 * al256(4 * nn);
    const unsigned grid = move_grid(nnz);
    invert_kernel<<<grid, MOVE_THREADS, 0, stream>>>(nnz, perm, inv);
    SBLAS_CUDA_TRY(cudaGetLastError());
    StageOp op;
    op.key_in = inv;
    op.key_out = slot_row;
    op.pos_out = reinterpret_cast<int *>(w + L.dst);
    rc = bsort::scatter_pass(op, nnz, sp.bits, sp.nb, pass_work, stream);
    if (rc != SBLAS_OK) return rc;
    const long long nt = stage_tiles(nnz);
    const size_t nruns = (size_t)nt * (size_t)sp.used;
    int *run_first = reinterpret_cast<int *>(w + L.runs);
    stage_runs_kernel<<<(unsigned)std::min<long long>((nruns + 255) / 256, 8LL * device_num_sms()),
                        256, 0, stream>>>(
        nnz, (int)nt, sp.used, sp.nb, static_cast<const int *>(pass_work), run_first,
        reinterpret_cast<unsigned short *>(w + L.runs + al256(4 * nruns)));
    SBLAS_CUDA_TRY(cudaGetLastError());
    invert_kernel<<<grid, MOVE_THREADS, 0, stream>>>(nnz, slot_row, perm);
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

int launch_csc_bind_values(int m, int n, long long nnz, const double *val, void *work,
                           size_t work_bytes, bool staged, cudaStream_t stream)
{
    if (m <= 0 || nnz <= 0) return SBLAS_OK;
    if (!check_work(m, n, nnz, work, work_bytes)) return SBLAS_ERR_ARG;
    const CscLayout L = csc_layout(m, n, nnz);
    unsigned char *w = static_cast<unsigned char *>(work);
    const int *perm = reinterpret_cast<const int *>(w + L.perm);
    double *rval = reinterpret_cast<double *>(w + L.val);
    const unsigned grid = move_grid(nnz);
    const StagePlan sp = stage_plan(nnz);
    if (staged && sp.used > 1) {
        double *stage = reinterpret_cast<double *>(w + L.scratch);
        const size_t nruns = (size_t)stage_tiles(nnz) * (size_t)sp.used;
        stage_scatter_kernel<<<(unsigned)stage_tiles(nnz), MOVE_THREADS, 0, stream>>>(
            nnz, sp.bits, sp.used, reinterpret_cast<const int *>(w + L.dst),
            reinterpret_cast<const int *>(w + L.runs),
            reinterpret_cast<const unsigned short *>(w + L.runs + al256(4 * nruns)), val, stage);
        SBLAS_CUDA_TRY(cudaGetLastError());
        gather_values_kernel<<<grid, MOVE_THREADS, 0, stream>>>(nnz, perm, stage, rval);
    } else {
        gather_values_kernel<<<grid, MOVE_THREADS, 0, stream>>>(nnz, perm, val, rval);
    }
    SBLAS_CUDA_TRY(cudaGetLastError());
    return SBLAS_OK;
}

int launch_cscmv_analysed(int m, int n, long long nnz, double alpha, const double *val,
                          const double *x, double beta, double *y, void *work,
                          size_t work_bytes, bool staged, cudaStream_t stream)
{
    if (m < 0 || n < 0 || nnz < 0 || nnz > 0x7fffffffLL) {
        set_error(SBLAS_ERR_ARG, "bad sizes m=%d n=%d nnz=%lld", m, n, nnz);
        return SBLAS_ERR_ARG;
    }
    if (m == 0) return SBLAS_OK;
    if (nnz == 0 || n == 0) return launch_scale_y(m, beta, y, stream);
    if (!check_work(m, n, nnz, work, work_bytes)) return SBLAS_ERR_ARG;
    const CscLayout L = csc_layout(m, n, nnz);
    unsigned char *w = static_cast<unsigned char *>(work);
    double *rval = reinterpret_cast<double *>(w + L.val);
    if (val != nullptr) {   // new values: into row order (else the bound ones)
        const int rc = launch_csc_bind_values(m, n, nnz, val, work, work_bytes, staged, stream);
        if (rc != SBLAS_OK) return rc;
    }
    return launch_tile_spmv(m, n, nnz, alpha, rval, VAL_F64,
                            reinterpret_cast<const int *>(w + L.rowptr),
                            reinterpret_cast<const int *>(w + L.col), x, beta, y, kCscSigma,
                            w + L.tile, stream, true);
}

int launch_cscmv(int m, int n, long long nnz, double alpha, const double *val,
                 const int *colptr, const int *rowidx, const double *x, double beta, double *y,
                 void *work, size_t work_bytes, cudaStream_t stream)
{
    // one product per analysis: the direct gather (staging indices would
    // cost more to build than they save once)
    const int rc = launch_csc_analyse(m, n, nnz, colptr, rowidx, work, work_bytes, false, stream);
    if (rc != SBLAS_OK) return rc;
    return launch_cscmv_analysed(m, n, nnz, alpha, val, x, beta, y, work, work_bytes, false,
                                 stream);
}

void *csc_tile_workspace(void *work, int m, int n, long long nnz)
{
    return static_cast<unsigned char *>(work) + csc_layout(m, n, nnz).tile;
}

}  // namespace sblas
