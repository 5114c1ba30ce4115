"""Device-side SpMV on torch tensors through the C ABI (include/sblas_gb300.h).

torch only provides device memory and the current CUDA stream; the work is
done by libsblas_gb300.so.  Nothing here falls back to torch or the CPU: a
missing library, a CPU tensor or a library error raises.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib

KERNEL_ROWSPLIT, KERNEL_MERGEPATH, KERNEL_CSR5 = 1, 2, 3
VAL_F64, VAL_F32, VAL_PATTERN = 0, 1, 2


def _stream_ptr(dev: torch.device) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _ptr(t: torch.Tensor | None) -> C.c_void_p:
    return C.c_void_p(t.data_ptr() if t is not None else 0)


def _require_cuda(*ts: torch.Tensor | None) -> torch.device:
    dev = None
    for t in ts:
        if t is None:
            continue
        if not t.is_cuda:
            raise ValueError("sblas ops take CUDA tensors (no CPU path)")
        if not t.is_contiguous():
            raise ValueError("sblas ops take contiguous tensors")
        dev = t.device if dev is None else dev
        if t.device != dev:
            raise ValueError("all tensors must be on one device")
    return dev


def workspace_bytes(nnz: int, sigma: int = 0) -> int:
    return int(_lib.load().sblas_tile_workspace_bytes(nnz, sigma))


def default_sigma(m: int, nnz: int) -> int:
    return int(_lib.load().sblas_default_sigma(m, nnz))


def compiled_sigmas() -> list[int]:
    lib = _lib.load()
    return [lib.sblas_tile_sigma_at(i) for i in range(lib.sblas_tile_sigma_count())]


def csrmv(rowptr: torch.Tensor, col: torch.Tensor, val: torch.Tensor | None, x: torch.Tensor,
          y: torch.Tensor, alpha: float = 1.0, beta: float = 0.0, n: int | None = None,
          kernel: int = KERNEL_MERGEPATH, sigma: int = 0,
          work: torch.Tensor | None = None) -> torch.Tensor:
    """y = alpha*A*x + beta*y in place (A in CSR, int32 indices).

    val: float64 (FP64 form), float32 (FP32 values, FP64 sums) or None
    (pattern-only: every stored entry is 1.0).  work: optional uint8 device
    buffer of workspace_bytes(nnz, sigma) bytes (needed for graph capture).
    """
    dev = _require_cuda(rowptr, col, val, x, y, work)
    if rowptr.dtype != torch.int32 or col.dtype != torch.int32:
        raise TypeError("rowptr and col must be int32")
    if x.dtype != torch.float64 or y.dtype != torch.float64:
        raise TypeError("x and y must be float64")
    if val is None:
        vk = VAL_PATTERN
    elif val.dtype == torch.float64:
        vk = VAL_F64
    elif val.dtype == torch.float32:
        vk = VAL_F32
    else:
        raise TypeError("val must be float64, float32 or None")
    m = rowptr.numel() - 1
    nnz = col.numel()
    if n is None:
        n = x.numel()
    if y.numel() != m or x.numel() < n:
        raise ValueError("shape mismatch")
    wb = work.numel() * work.element_size() if work is not None else 0
    lib = _lib.load()
    with torch.cuda.device(dev):
        rc = lib.sblas_dcsrmv(kernel, m, n, nnz, float(alpha), _ptr(val), vk, _ptr(rowptr),
                              _ptr(col), _ptr(x), float(beta), _ptr(y), sigma, _ptr(work), wb,
                              _stream_ptr(dev))
    _lib.check(rc)
    return y


def coomv(row: torch.Tensor, col: torch.Tensor, val: torch.Tensor, x: torch.Tensor,
          y: torch.Tensor, alpha: float = 1.0, beta: float = 0.0, n: int | None = None,
          rowptr_work: torch.Tensor | None = None, sigma: int = 0) -> torch.Tensor:
    """y = alpha*A*x + beta*y with A in row-sorted COO (int32)."""
    dev = _require_cuda(row, col, val, x, y)
    m = y.numel()
    if rowptr_work is None:
        rowptr_work = torch.empty(m + 1, dtype=torch.int32, device=dev)
    lib = _lib.load()
    with torch.cuda.device(dev):
        rc = lib.sblas_dcoomv(m, n if n is not None else x.numel(), col.numel(), float(alpha),
                              _ptr(val), _ptr(row), _ptr(col), _ptr(x), float(beta), _ptr(y),
                              _ptr(rowptr_work), sigma, C.c_void_p(0), 0, _stream_ptr(dev))
    _lib.check(rc)
    return y


def csc_to_csr(m: int, n: int, colptr: torch.Tensor, rowidx: torch.Tensor,
               val: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Device CSC -> CSR (stable; columns ascending inside each row)."""
    dev = _require_cuda(colptr, rowidx, val)
    nnz = rowidx.numel()
    lib = _lib.load()
    wb = int(lib.sblas_csc_to_csr_workspace_bytes(m, n, nnz))
    work = torch.empty(max(wb, 1), dtype=torch.uint8, device=dev)
    rowptr = torch.empty(m + 1, dtype=torch.int32, device=dev)
    col = torch.empty(nnz, dtype=torch.int32, device=dev)
    oval = torch.empty(nnz, dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        rc = lib.sblas_csc_to_csr(m, n, nnz, _ptr(val), _ptr(colptr), _ptr(rowidx), _ptr(oval),
                                  _ptr(rowptr), _ptr(col), _ptr(work), wb, _stream_ptr(dev))
    _lib.check(rc)
    return rowptr, col, oval


def cscmv(colptr: torch.Tensor, rowidx: torch.Tensor, val: torch.Tensor, x: torch.Tensor,
          y: torch.Tensor, alpha: float = 1.0, beta: float = 0.0) -> torch.Tensor:
    """y = alpha*A*x + beta*y with A in CSC: device transpose to CSR, then the
    atomic-free tile kernel."""
    m = y.numel()
    n = colptr.numel() - 1
    rp, c, v = csc_to_csr(m, n, colptr, rowidx, val)
    return csrmv(rp, c, v, x, y, alpha, beta, n=n)


class CsrPlan:
    """A CSR matrix analysed once for repeated products (kernel 2 or 3).

    The tile partition of the row pointer is computed at construction
    (sblas_csr_analyse) into a workspace owned by the plan; each call runs
    only the tile kernel and the carry fix-up (sblas_dcsrmv_analysed), does
    not allocate and can be captured in a CUDA graph.
    """

    def __init__(self, rowptr: torch.Tensor, col: torch.Tensor, val: torch.Tensor | None,
                 n: int | None = None, kernel: int = KERNEL_MERGEPATH, sigma: int = 0):
        dev = _require_cuda(rowptr, col, val)
        if kernel not in (KERNEL_MERGEPATH, KERNEL_CSR5):
            raise ValueError("plans use the tile kernels (2 or 3)")
        lib = _lib.load()
        self.rowptr, self.col, self.val = rowptr, col, val
        self.m = rowptr.numel() - 1
        self.nnz = col.numel()
        self.n = int(n) if n is not None else None
        self.kernel = kernel
        if sigma <= 0:
            sigma = (lib.sblas_csr5_sigma(self.m, self.nnz) if kernel == KERNEL_CSR5
                     else lib.sblas_default_sigma(self.m, self.nnz))
        self.sigma = int(sigma)
        if val is None:
            self.vk = VAL_PATTERN
        elif val.dtype == torch.float64:
            self.vk = VAL_F64
        elif val.dtype == torch.float32:
            self.vk = VAL_F32
        else:
            raise TypeError("val must be float64, float32 or None")
        self.work_bytes = int(lib.sblas_tile_workspace_bytes(self.nnz, self.sigma))
        self.work = torch.empty(self.work_bytes, dtype=torch.uint8, device=dev)
        self.device = dev
        with torch.cuda.device(dev):
            rc = lib.sblas_csr_analyse(kernel, self.m, self.nnz, _ptr(rowptr), self.sigma,
                                       _ptr(self.work), self.work_bytes, _stream_ptr(dev))
        _lib.check(rc)

    def __call__(self, x: torch.Tensor, y: torch.Tensor, alpha: float = 1.0,
                 beta: float = 0.0) -> torch.Tensor:
        n = self.n if self.n is not None else x.numel()
        lib = _lib.load()
        rc = lib.sblas_dcsrmv_analysed(self.kernel, self.m, n, self.nnz, float(alpha),
                                       _ptr(self.val), self.vk, _ptr(self.rowptr), _ptr(self.col),
                                       _ptr(x), float(beta), _ptr(y), self.sigma, _ptr(self.work),
                                       self.work_bytes, _stream_ptr(self.device))
        _lib.check(rc)
        return y
