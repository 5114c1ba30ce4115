// Host side of the batched SpMM (include/sblas_gb300.h, sblas_batch_*):
// plan creation (descriptor upload, unit partition, persistent grid), runs,
// and the per-K dispatch into the compiled shapes (spmm_k*.cu).
#include <climits>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "spmm_batched.cuh"

namespace sblas {
namespace batch {
cudaError_t dispatch_k1(Op, int, int, const Args *, int, int, int *, cudaStream_t);
cudaError_t dispatch_k2(Op, int, int, const Args *, int, int, int *, cudaStream_t);
cudaError_t dispatch_k4(Op, int, int, const Args *, int, int, int *, cudaStream_t);
cudaError_t dispatch_k8(Op, int, int, const Args *, int, int, int *, cudaStream_t);
cudaError_t dispatch_k16(Op, int, int, const Args *, int, int, int *, cudaStream_t);

namespace {

cudaError_t dispatch(Op op, int K, int S, int VK, const Args *a, int nunits, int grid,
                     int *grid_out, cudaStream_t st)
{
    switch (K) {
    case 1: return dispatch_k1(op, S, VK, a, nunits, grid, grid_out, st);
    case 2: return dispatch_k2(op, S, VK, a, nunits, grid, grid_out, st);
    case 4: return dispatch_k4(op, S, VK, a, nunits, grid, grid_out, st);
    case 8: return dispatch_k8(op, S, VK, a, nunits, grid, grid_out, st);
    case 16: return dispatch_k16(op, S, VK, a, nunits, grid, grid_out, st);
    default: return cudaErrorInvalidValue;
    }
}

// ---- unit partition (analysis): matrix and first row of every unit --------
__global__ void batch_partition_kernel(const Mat *mats, int nmat, int *unit_mat, int *unit_row,
                                       int nunits, int unit_nnz)
{
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nunits;
         u += gridDim.x * blockDim.x) {
        int lo = 0, hi = nmat - 1;            // last matrix with unit0 <= u
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (mats[mid].unit0 <= u) lo = mid; else hi = mid - 1;
        }
        const Mat *M = mats + lo;
        unit_mat[u] = lo;
        const int lu = u - M->unit0;
        int r = 0;
        if (lu > 0) {
            const int s = lu * unit_nnz;        // row containing nonzero s
            int a = 0, b = M->m - 1;
            while (a < b) {
                const int mid = (a + b + 1) >> 1;
                if (__ldg(M->rowptr + mid) <= s) a = mid; else b = mid - 1;
            }
            r = a;
        }
        unit_row[u] = r;
    }
}

bool k_compiled(int k) { return k == 1 || k == 2 || k == 4 || k == 8 || k == 16; }
bool s_compiled(int s) { return s == 4 || s == 8 || s == 16 || s == 32; }

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

size_t up256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace
}  // namespace batch
}  // namespace sblas

struct sblas_batch_plan {
    int nmat;
    int k;
    int val_kind;
    int s;
    int grid;
    int nunits;
    int device;
    void *mem;
    size_t mem_bytes;
    sblas::batch::Args args;
    // one right-hand side, contiguous x and y, no row list or value
    // permutation: sblas_batch_spmm runs the tile kernel over all matrices
    // in one launch (multi-matrix tiles) instead of the warp-unit kernel
    int multi;
    void *multi_mem;
    size_t multi_bytes;
    sblas::MultiTileLaunch multi_launch;
};

namespace sblas {
namespace batch {
namespace {

// Tiles, partitions and carries of the multi-matrix tile launch of a plan.
int build_multi(sblas_batch_plan *p, const sblas_batch_matrix *mats, cudaStream_t st)
{
    const int nmat = p->nmat;
    std::vector<int> tile0s(nmat + 1), part_off(nmat);
    long long tiles = 0, parts = 0;
    for (int i = 0; i < nmat; ++i) {
        tile0s[i] = (int)tiles;
        part_off[i] = (int)parts;
        const long long nt = (long long)multi_tile_count(mats[i].nnz);
        tiles += nt;
        parts += nt + 1;
        if (tiles > INT_MAX / 2 || parts > INT_MAX / 2) {
            set_error(SBLAS_ERR_ARG, "batch too large for one launch (%lld tiles)", tiles);
            return SBLAS_ERR_ARG;
        }
    }
    tile0s[nmat] = (int)tiles;
    const size_t b_mats = up256(multi_mat_bytes() * (size_t)nmat);
    const size_t b_t0 = up256(sizeof(int) * (size_t)(nmat + 1));
    const size_t b_part = up256(sizeof(int) * (size_t)parts);
    const size_t b_carry = up256(sizeof(double) * (size_t)tiles);
    const size_t total = b_mats + b_t0 + b_part + b_carry + 256;
    cudaError_t e = cudaMalloc(&p->multi_mem, total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        p->multi_mem = nullptr;
        set_error(SBLAS_ERR_ALLOC, "plan allocation of %zu bytes: %s", total,
                  cudaGetErrorString(e));
        return SBLAS_ERR_ALLOC;
    }
    p->multi_bytes = total;
    unsigned char *b = static_cast<unsigned char *>(p->multi_mem);
    std::vector<unsigned char> hm(multi_mat_bytes() * (size_t)nmat);
    for (int i = 0; i < nmat; ++i) {
        const sblas_batch_matrix &q = mats[i];
        fill_multi_mat(hm.data() + multi_mat_bytes() * i, q.val, q.rowptr, q.col, q.x, q.y,
                       q.nnz, q.m, tile0s[i], part_off[i], q.alpha, q.beta, p->val_kind);
    }
    MultiTileLaunch &L = p->multi_launch;
    L.mats = b;
    L.tile0s = reinterpret_cast<const int *>(b + b_mats);
    L.nmat = nmat;
    L.ntiles = (int)tiles;
    int *part = reinterpret_cast<int *>(b + b_mats + b_t0);
    L.part = part;
    L.carry = reinterpret_cast<double *>(b + b_mats + b_t0 + b_part);
    L.status = reinterpret_cast<int *>(b + b_mats + b_t0 + b_part + b_carry);
    e = cudaMemcpyAsync(b, hm.data(), hm.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b + b_mats, tile0s.data(), sizeof(int) * (size_t)(nmat + 1),
                            cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        set_error(SBLAS_ERR_CUDA, "plan upload: %s", cudaGetErrorString(e));
        return SBLAS_ERR_CUDA;
    }
    // every matrix's tile partition; a matrix without nonzeros is one tile
    // owning all its rows
    std::vector<int> empty_part;
    for (int i = 0; i < nmat; ++i) {
        const sblas_batch_matrix &q = mats[i];
        if (q.nnz > 0 && q.m > 0) {
            const int rc = launch_tile_partition(q.m, q.nnz, q.rowptr, multi_tile_sigma(),
                                                 part + part_off[i], st);
            if (rc != SBLAS_OK) return rc;
        } else {
            empty_part.push_back(i);
        }
    }
    std::vector<int> pairs(2 * empty_part.size());
    for (size_t j = 0; j < empty_part.size(); ++j) {
        pairs[2 * j] = 0;
        pairs[2 * j + 1] = mats[empty_part[j]].m;
        e = cudaMemcpyAsync(part + part_off[empty_part[j]], pairs.data() + 2 * j, 2 * sizeof(int),
                            cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            set_error(SBLAS_ERR_CUDA, "plan upload: %s", cudaGetErrorString(e));
            return SBLAS_ERR_CUDA;
        }
    }
    // the host vectors above must outlive the copies
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error(SBLAS_ERR_CUDA, "plan analysis: %s", cudaGetErrorString(e));
        return SBLAS_ERR_CUDA;
    }
    p->multi = 1;
    return SBLAS_OK;
}

}  // namespace
}  // namespace batch
}  // namespace sblas

using namespace sblas;
using namespace sblas::batch;

extern "C" {

int sblas_batch_default_s(int k)
{
    // nonzeros per lane: long chunks for one right-hand side (more gathers
    // in flight per lane), shorter ones as the row of X grows
    switch (k) {
    case 1: return 16;
    case 2: return 16;
    case 4: return 8;
    case 8: return 8;
    case 16: return 4;
    default: return 0;
    }
}

int sblas_batch_plan_create(int nmat, const sblas_batch_matrix *mats, int k, int val_kind, int s,
                            void *stream, sblas_batch_plan **plan_out)
{
    clear_error();
    if (plan_out == nullptr || mats == nullptr || nmat < 1) {
        set_error(SBLAS_ERR_ARG, "sblas_batch_plan_create: need nmat >= 1, mats and plan");
        return SBLAS_ERR_ARG;
    }
    *plan_out = nullptr;
    if (!k_compiled(k)) {
        set_error(SBLAS_ERR_UNSUPPORTED, "k = %d not compiled (1, 2, 4, 8, 16)", k);
        return SBLAS_ERR_UNSUPPORTED;
    }
    if (s == 0) s = sblas_batch_default_s(k);
    if (!s_compiled(s)) {
        set_error(SBLAS_ERR_UNSUPPORTED, "s = %d not compiled (4, 8, 16, 32)", s);
        return SBLAS_ERR_UNSUPPORTED;
    }
    if (val_kind < SBLAS_VAL_F64 || val_kind > SBLAS_VAL_PATTERN) {
        set_error(SBLAS_ERR_ARG, "unknown value kind %d", val_kind);
        return SBLAS_ERR_ARG;
    }
    const long long unit = 32LL * s;
    std::vector<Mat> dm(nmat);
    long long units = 0;
    for (int i = 0; i < nmat; ++i) {
        const sblas_batch_matrix &q = mats[i];
        if (q.m < 0 || q.n < 0 || q.nnz < 0 || q.nnz > INT_MAX) {
            set_error(SBLAS_ERR_ARG, "matrix %d: bad sizes m=%d n=%d nnz=%lld", i, q.m, q.n, q.nnz);
            return SBLAS_ERR_ARG;
        }
        if (q.rowptr == nullptr || ((q.m > 0 || q.row_ids) && q.y == nullptr) ||
            (q.nnz > 0 && (q.col == nullptr || q.x == nullptr ||
                           (val_kind != SBLAS_VAL_PATTERN && q.val == nullptr)))) {
            set_error(SBLAS_ERR_ARG, "matrix %d: null device pointer", i);
            return SBLAS_ERR_ARG;
        }
        if (q.ldx < k || q.ldy < k ||
            (k >= 2 && ((q.ldx & 1) || (q.ldy & 1) || !aligned16(q.x) || !aligned16(q.y)))) {
            set_error(SBLAS_ERR_ALIGN,
                      "matrix %d: need ldx, ldy >= k, and for k >= 2 even strides and "
                      "16-byte aligned x, y", i);
            return SBLAS_ERR_ALIGN;
        }
        Mat &d = dm[i];
        d.val = q.val;
        d.rowptr = q.rowptr;
        d.col = q.col;
        d.x = q.x;
        d.y = q.y;
        d.nnz = q.nnz;
        d.m = q.m;
        d.n = q.n;
        d.ldx = q.ldx;
        d.ldy = q.ldy;
        d.alpha = q.alpha;
        d.beta = q.beta;
        d.row_ids = q.row_ids;
        d.val_perm = q.val_perm;
        const long long nu = q.nnz > 0 ? (q.nnz + unit - 1) / unit : 1;
        d.unit0 = (int)units;
        d.nunits = (int)nu;
        units += nu;
        if (units > INT_MAX / 2) {
            set_error(SBLAS_ERR_ARG, "batch too large (%lld units)", units);
            return SBLAS_ERR_ARG;
        }
    }
    const int nunits = (int)units;
    // device memory: descriptors | unit_mat | unit_row | head_row | tail_row | head_val | tail_val
    const size_t b_mats = up256(sizeof(Mat) * nmat);
    const size_t b_int = up256(sizeof(int) * (size_t)nunits);
    const size_t b_val = up256(sizeof(double) * (size_t)nunits * k);
    const size_t total = b_mats + 4 * b_int + 2 * b_val;
    sblas_batch_plan *p = static_cast<sblas_batch_plan *>(std::calloc(1, sizeof(sblas_batch_plan)));
    if (!p) {
        set_error(SBLAS_ERR_ALLOC, "host allocation failed");
        return SBLAS_ERR_ALLOC;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaGetDevice(&p->device);
    if (e == cudaSuccess) e = cudaMalloc(&p->mem, total);
    if (e != cudaSuccess) {
        set_error(e == cudaErrorMemoryAllocation ? SBLAS_ERR_ALLOC : SBLAS_ERR_CUDA,
                  "plan allocation of %zu bytes: %s", total, cudaGetErrorString(e));
        std::free(p);
        return e == cudaErrorMemoryAllocation ? SBLAS_ERR_ALLOC : SBLAS_ERR_CUDA;
    }
    p->mem_bytes = total;
    p->nmat = nmat;
    p->k = k;
    p->val_kind = val_kind;
    p->s = s;
    p->nunits = nunits;
    unsigned char *base = static_cast<unsigned char *>(p->mem);
    Args &a = p->args;
    a.mats = reinterpret_cast<const Mat *>(base);
    a.nmat = nmat;
    a.unit_mat = reinterpret_cast<const int *>(base + b_mats);
    a.unit_row = reinterpret_cast<const int *>(base + b_mats + b_int);
    a.head_row = reinterpret_cast<int *>(base + b_mats + 2 * b_int);
    a.tail_row = reinterpret_cast<int *>(base + b_mats + 3 * b_int);
    a.head_val = reinterpret_cast<double *>(base + b_mats + 4 * b_int);
    a.tail_val = reinterpret_cast<double *>(base + b_mats + 4 * b_int + b_val);
    a.nunits = nunits;
    a.override_xy = 0;
    e = cudaMemcpyAsync(base, dm.data(), sizeof(Mat) * nmat, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const int pgrid = (nunits + 255) / 256 < 4096 ? (nunits + 255) / 256 : 4096;
        batch_partition_kernel<<<pgrid, 256, 0, st>>>(a.mats, nmat, const_cast<int *>(a.unit_mat),
                                                      const_cast<int *>(a.unit_row), nunits,
                                                      (int)unit);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = dispatch(Op::GRID, k, s, val_kind, nullptr, nunits, 0, &p->grid, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error(SBLAS_ERR_CUDA, "plan analysis: %s", cudaGetErrorString(e));
        cudaFree(p->mem);
        std::free(p);
        return SBLAS_ERR_CUDA;
    }
    bool multi = (k == 1);
    for (int i = 0; i < nmat && multi; ++i)
        multi = mats[i].row_ids == nullptr && mats[i].val_perm == nullptr && mats[i].ldx == 1 &&
                mats[i].ldy == 1;
    if (multi) {
        const int rc = build_multi(p, mats, st);
        if (rc != SBLAS_OK) {
            if (p->multi_mem) cudaFree(p->multi_mem);
            cudaFree(p->mem);
            std::free(p);
            return rc;
        }
    }
    *plan_out = p;
    return SBLAS_OK;
}

int sblas_batch_plan_destroy(sblas_batch_plan *plan)
{
    clear_error();
    if (!plan) return SBLAS_OK;
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != plan->device) cudaSetDevice(plan->device);
    cudaError_t e = cudaFree(plan->mem);
    if (plan->multi_mem) {
        const cudaError_t e2 = cudaFree(plan->multi_mem);
        if (e == cudaSuccess) e = e2;
    }
    if (cur >= 0 && cur != plan->device) cudaSetDevice(cur);
    std::free(plan);
    if (e != cudaSuccess) {
        set_error(SBLAS_ERR_CUDA, "cudaFree: %s", cudaGetErrorString(e));
        return SBLAS_ERR_CUDA;
    }
    return SBLAS_OK;
}

int sblas_batch_plan_info(const sblas_batch_plan *plan, long long *units, int *s,
                          size_t *device_bytes)
{
    clear_error();
    if (!plan) {
        set_error(SBLAS_ERR_ARG, "null plan");
        return SBLAS_ERR_ARG;
    }
    if (units) *units = plan->nunits;
    if (s) *s = plan->s;
    if (device_bytes) *device_bytes = plan->mem_bytes + plan->multi_bytes;
    return SBLAS_OK;
}

int sblas_batch_spmm(const sblas_batch_plan *plan, void *stream)
{
    clear_error();
    if (!plan) {
        set_error(SBLAS_ERR_ARG, "null plan");
        return SBLAS_ERR_ARG;
    }
    if (plan->multi)
        return launch_multi_tile_spmv(plan->multi_launch, plan->val_kind,
                                      static_cast<cudaStream_t>(stream));
    const cudaError_t e = dispatch(Op::SPMM, plan->k, plan->s, plan->val_kind, &plan->args,
                                   plan->nunits, plan->grid, nullptr,
                                   static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        set_error(SBLAS_ERR_CUDA, "batched SpMM launch: %s", cudaGetErrorString(e));
        return SBLAS_ERR_CUDA;
    }
    return SBLAS_OK;
}

int sblas_batch_spmm_xy(const sblas_batch_plan *plan, const void *val, const double *x, int ldx,
                        double *y, int ldy, double alpha, double beta, void *stream)
{
    clear_error();
    if (!plan || plan->nmat != 1) {
        set_error(SBLAS_ERR_ARG, "sblas_batch_spmm_xy needs a single-matrix plan");
        return SBLAS_ERR_ARG;
    }
    const int k = plan->k;
    if (x == nullptr || y == nullptr || ldx < k || ldy < k ||
        (k >= 2 && ((ldx & 1) || (ldy & 1) || !aligned16(x) || !aligned16(y)))) {
        set_error(SBLAS_ERR_ALIGN,
                  "need non-null x, y, ldx, ldy >= k, and for k >= 2 even strides and "
                  "16-byte aligned x, y");
        return SBLAS_ERR_ALIGN;
    }
    Args a = plan->args;
    a.override_xy = 1;
    a.val = val;
    a.x = x;
    a.y = y;
    a.ldx = ldx;
    a.ldy = ldy;
    a.alpha = alpha;
    a.beta = beta;
    const cudaError_t e = dispatch(Op::SPMM, k, plan->s, plan->val_kind, &a, plan->nunits,
                                   plan->grid, nullptr, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        set_error(SBLAS_ERR_CUDA, "batched SpMM launch: %s", cudaGetErrorString(e));
        return SBLAS_ERR_CUDA;
    }
    return SBLAS_OK;
}

int sblas_batch_sddmm(const sblas_batch_plan *plan, const double *g, int ldg, const double *x,
                      int ldx, void *dval, void *stream)
{
    clear_error();
    if (!plan || plan->nmat != 1) {
        set_error(SBLAS_ERR_ARG, "sblas_batch_sddmm needs a single-matrix plan");
        return SBLAS_ERR_ARG;
    }
    if (plan->val_kind == SBLAS_VAL_PATTERN) {
        set_error(SBLAS_ERR_UNSUPPORTED, "a pattern-only matrix has no values to differentiate");
        return SBLAS_ERR_UNSUPPORTED;
    }
    const int k = plan->k;
    if (g == nullptr || x == nullptr || dval == nullptr || ldg < k || ldx < k ||
        (k >= 2 && ((ldx & 1) || (ldg & 1) || !aligned16(x) || !aligned16(g)))) {
        set_error(SBLAS_ERR_ALIGN,
                  "need non-null g, x, dval, ldg, ldx >= k, and for k >= 2 even strides and "
                  "16-byte aligned g, x");
        return SBLAS_ERR_ALIGN;
    }
    Args a = plan->args;
    a.override_xy = 1;
    a.x = x;
    a.ldx = ldx;
    a.g = g;
    a.ldg = ldg;
    a.dval = dval;
    const long long want = ((long long)plan->nunits + NW - 1) / NW;
    const long long cap = 16LL * device_num_sms();
    const int grid = (int)(want < 1 ? 1 : (want < cap ? want : cap));
    const cudaError_t e = dispatch(Op::SDDMM, k, plan->s, plan->val_kind, &a, plan->nunits, grid,
                                   nullptr, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        set_error(SBLAS_ERR_CUDA, "sampled product launch: %s", cudaGetErrorString(e));
        return SBLAS_ERR_CUDA;
    }
    return SBLAS_OK;
}

}  // extern "C"
