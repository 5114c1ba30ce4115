"""GB300-native FP64 sparse matrix-vector multiply behind the C entry points
of PNNL's multi-GPU Sparse-BLAS (spMV_mgpu_baseline / v1 / v2, ngpu = 1).

  libsblas_gb300.so   hand-written sm_103a CUDA kernels + C ABI (csrc/)
  api                 Python mirror of the reference's entry points (host arrays)
  ops                 device-side calls on torch tensors (current stream), plans
                      for repeated products, the batched multi-matrix SpMM,
                      SpMSpV (x-zero filter on the device)
  mmio                MatrixMarket files to COO / CSR (multi-threaded reader)
  autograd            Y = A X as a torch.autograd.Function with adjoint kernels
  tune                measured choice of tile shapes (sigma, nonzeros per lane)
  synth               seeded synthetic matrices of the benchmark shapes
"""
from ._lib import SblasError, SpmvRet, load  # noqa: F401

__version__ = "0.1.0"
