// Batched SpMM shapes with 2 right-hand side(s) per matrix (one translation
// unit per K so that the shapes compile in parallel).
#include "spmm_batched.cuh"

namespace sblas {
namespace batch {

cudaError_t dispatch_k2(Op op, int S, int VK, const Args *a, int nunits, int grid,
                        int *grid_out, cudaStream_t stream)
{
    return dispatch_k<2>(op, S, VK, a, nunits, grid, grid_out, stream);
}

}  // namespace batch
}  // namespace sblas
