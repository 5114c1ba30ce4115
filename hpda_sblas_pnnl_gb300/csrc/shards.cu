// Multi-device form of the reference's nnz-balanced split (host code only).
//
// The reference's spMV_mgpu_v1 cuts the nonzeros of a CSR matrix into ngpu
// equal ranges, finds the rows holding the cuts, flags rows split by a cut
// (src/dspmv_mgpu_v1.cu:120-152), gives every part its own row pointer with
// the first and last rows clipped to the part (:183-193), runs each part on
// its GPU and merges the parts' row ranges back into y, adding the two
// halves of every split row and removing the second beta*y0 term
// (:304-319).  Inside one GPU this library applies the same decomposition
// per tile; these functions are the decomposition across devices (one
// process per GPU, the parts exchanged by the caller, e.g. with
// torch.distributed), computing exactly the reference's cut points and
// merge order so that the merged y equals the reference's bit for bit
// given the same per-part results.
#include <cstring>
#include <vector>

#include "../../include/spmv_kernel.h"
#include "sblas_internal.h"

using namespace sblas;

extern "C" {

int sblas_nnz_partition(int m, long long nnz, const int *rowptr, int nparts,
                        sblas_nnz_part *parts)
{
    clear_error();
    if (m <= 0 || nnz <= 0 || nnz > 0x7fffffffLL || rowptr == nullptr || parts == nullptr ||
        nparts <= 0) {
        set_error(SBLAS_ERR_ARG, "sblas_nnz_partition: bad arguments (m=%d nnz=%lld nparts=%d)",
                  m, nnz, nparts);
        return SBLAS_ERR_ARG;
    }
    if (nnz < nparts) {
        set_error(SBLAS_ERR_ARG, "sblas_nnz_partition: %lld nonzeros cannot fill %d parts", nnz,
                  nparts);
        return SBLAS_ERR_ARG;
    }
    if ((long long)rowptr[m] != nnz || rowptr[0] != 0) {
        set_error(SBLAS_ERR_ARG, "sblas_nnz_partition: rowptr[0] must be 0 and rowptr[m] = nnz");
        return SBLAS_ERR_ARG;
    }
    for (int i = 0; i < nparts; ++i) {
        sblas_nnz_part &p = parts[i];
        // floor(i*nnz/ngpu) (:122-129), in 64-bit: the reference's int product
        // overflows once nnz*ngpu passes 2^31
        p.start_idx = (int)((long long)i * nnz / nparts);
        p.end_idx = (int)((long long)(i + 1) * nnz / nparts) - 1;
        p.start_row = get_row_from_index(m, const_cast<int *>(rowptr), p.start_idx);
        p.end_row = get_row_from_index(m, const_cast<int *>(rowptr), p.end_idx);
        p.start_flag = p.start_idx > rowptr[p.start_row] ? 1 : 0;   // :135-140
        p.end_flag = p.end_idx < rowptr[p.end_row + 1] - 1 ? 1 : 0;  // :145-150
        p.m = p.end_row - p.start_row + 1;
        p.nnz = p.end_idx - p.start_idx + 1;
    }
    return SBLAS_OK;
}

int sblas_part_rowptr(const int *rowptr, const sblas_nnz_part *part, int *out)
{
    clear_error();
    if (rowptr == nullptr || part == nullptr || out == nullptr || part->m <= 0) {
        set_error(SBLAS_ERR_ARG, "sblas_part_rowptr: bad arguments");
        return SBLAS_ERR_ARG;
    }
    // :183-193: first entry 0, last entry the part's nonzero count, inner
    // rows rebased to the part's first nonzero
    out[0] = 0;
    out[part->m] = part->nnz;
    for (int j = 1; j < part->m; ++j) out[j] = rowptr[part->start_row + j] - part->start_idx;
    return SBLAS_OK;
}

int sblas_merge_parts(int nparts, const sblas_nnz_part *parts, const double *const *part_y,
                      double beta, double *y)
{
    clear_error();
    if (nparts <= 0 || parts == nullptr || part_y == nullptr || y == nullptr) {
        set_error(SBLAS_ERR_ARG, "sblas_merge_parts: bad arguments");
        return SBLAS_ERR_ARG;
    }
    for (int d = 0; d < nparts; ++d)
        if (part_y[d] == nullptr || parts[d].m <= 0) {
            set_error(SBLAS_ERR_ARG, "sblas_merge_parts: part %d has no rows or no result", d);
            return SBLAS_ERR_ARG;
        }
    // the caller's y0 at every split row, taken before any part is copied in
    // (the reference's y2, :137)
    std::vector<double> y2((size_t)nparts, 0.0);
    for (int d = 0; d < nparts; ++d)
        if (parts[d].start_flag) y2[(size_t)d] = y[parts[d].start_row];
    // :304-319, in part order: copy the part's rows; a row split with the
    // previous part gets that part's value added back and the second
    // beta*y0 removed
    for (int d = 0; d < nparts; ++d) {
        const sblas_nnz_part &p = parts[d];
        double tmp = 0.0;
        if (p.start_flag) tmp = y[p.start_row];
        std::memcpy(y + p.start_row, part_y[d], sizeof(double) * (size_t)p.m);
        if (p.start_flag) {
            y[p.start_row] += tmp;
            const double twice = y2[(size_t)d] * beta;
            y[p.start_row] -= twice;
        }
    }
    return SBLAS_OK;
}

}  // extern "C"
