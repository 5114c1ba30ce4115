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


def _require_dtype(what: str, t: torch.Tensor | None, dtype: torch.dtype) -> None:
    if t is not None and t.dtype != dtype:
        raise TypeError(f"{what} must be {dtype} (got {t.dtype})")


def _require_len(what: str, t: torch.Tensor | None, need: int) -> None:
    """The kernels take bare pointers: an array shorter than the sizes say
    would be read past its end on the device."""
    if t is not None and t.numel() < need:
        raise ValueError(f"{what} holds {t.numel()} elements, {need} needed")


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
    _require_len("val", val, nnz)
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
    dev = _require_cuda(row, col, val, x, y, rowptr_work)
    for what, t, dt in (("row", row, torch.int32), ("col", col, torch.int32),
                        ("val", val, torch.float64), ("x", x, torch.float64),
                        ("y", y, torch.float64), ("rowptr_work", rowptr_work, torch.int32)):
        _require_dtype(what, t, dt)
    m = y.numel()
    n = n if n is not None else x.numel()
    _require_len("row", row, col.numel())
    _require_len("val", val, col.numel())
    _require_len("x", x, n)
    _require_len("rowptr_work", rowptr_work, m + 1)
    if rowptr_work is None:
        rowptr_work = torch.empty(m + 1, dtype=torch.int32, device=dev)
    lib = _lib.load()
    with torch.cuda.device(dev):
        rc = lib.sblas_dcoomv(m, n, col.numel(), float(alpha),
                              _ptr(val), _ptr(row), _ptr(col), _ptr(x), float(beta), _ptr(y),
                              _ptr(rowptr_work), sigma, C.c_void_p(0), 0, _stream_ptr(dev))
    _lib.check(rc)
    return y


def csc_to_csr(m: int, n: int, colptr: torch.Tensor, rowidx: torch.Tensor,
               val: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Device CSC -> CSR (stable; columns ascending inside each row)."""
    dev = _require_cuda(colptr, rowidx, val)
    _require_dtype("colptr", colptr, torch.int32)
    _require_dtype("rowidx", rowidx, torch.int32)
    _require_dtype("val", val, torch.float64)
    nnz = rowidx.numel()
    _require_len("colptr", colptr, n + 1)
    _require_len("val", val, nnz)
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


def cscmv_workspace_bytes(m: int, n: int, nnz: int) -> int:
    return int(_lib.load().sblas_cscmv_workspace_bytes(m, n, nnz))


def cscmv(colptr: torch.Tensor, rowidx: torch.Tensor, val: torch.Tensor, x: torch.Tensor,
          y: torch.Tensor, alpha: float = 1.0, beta: float = 0.0,
          work: torch.Tensor | None = None) -> torch.Tensor:
    """y = alpha*A*x + beta*y with A in CSC (sblas_dcscmv): the row-ordered
    structure by a stable bucket sort (inspector), then the values gathered
    into row order and the CSR tile kernel: atomic-free, bit-reproducible.
    work: optional uint8 device buffer of cscmv_workspace_bytes(m, n, nnz)."""
    dev = _require_cuda(colptr, rowidx, val, x, y, work)
    for what, t, dt in (("colptr", colptr, torch.int32), ("rowidx", rowidx, torch.int32),
                        ("val", val, torch.float64), ("x", x, torch.float64),
                        ("y", y, torch.float64)):
        _require_dtype(what, t, dt)
    m = y.numel()
    n = colptr.numel() - 1
    nnz = rowidx.numel()
    _require_len("val", val, nnz)
    _require_len("x", x, n)
    wb = work.numel() * work.element_size() if work is not None else 0
    lib = _lib.load()
    with torch.cuda.device(dev):
        rc = lib.sblas_dcscmv(m, n, nnz, float(alpha), _ptr(val), _ptr(colptr), _ptr(rowidx),
                              _ptr(x), float(beta), _ptr(y), _ptr(work), wb, _stream_ptr(dev))
    _lib.check(rc)
    return y


class CscPlan:
    """A CSC pattern (int32 colptr, rowidx) analysed once (sblas_csc_analyse:
    the row-ordered structure, the permutation to it, the staging indices
    of patterns above 2^22 entries and the tile partition, held in the
    plan's workspace); each call runs only the executor
    (sblas_dcscmv_analysed: the values moved into row order and the tile
    kernel), with the values, x and y given per call; bind() keeps one set
    of values in row order (calls with val=None then skip the move)."""

    def __init__(self, m: int, colptr: torch.Tensor, rowidx: torch.Tensor):
        dev = _require_cuda(colptr, rowidx)
        _require_dtype("colptr", colptr, torch.int32)
        _require_dtype("rowidx", rowidx, torch.int32)
        self.m, self.n, self.nnz = int(m), colptr.numel() - 1, rowidx.numel()
        self.colptr, self.rowidx, self.device = colptr, rowidx, dev
        lib = _lib.load()
        self.work_bytes = int(lib.sblas_cscmv_workspace_bytes(self.m, self.n, self.nnz))
        self.work = torch.empty(self.work_bytes, dtype=torch.uint8, device=dev)
        with torch.cuda.device(dev):
            rc = lib.sblas_csc_analyse(self.m, self.n, self.nnz, _ptr(colptr), _ptr(rowidx),
                                       _ptr(self.work), self.work_bytes, _stream_ptr(dev))
        _lib.check(rc)

    def bind(self, val: torch.Tensor) -> None:
        """Keeps these values (CSC order) in row order inside the plan: calls
        with val=None then use them and skip the per-call gather."""
        if _require_cuda(val) != self.device:
            raise ValueError("val must be on the plan's device")
        _require_dtype("val", val, torch.float64)
        _require_len("val", val, self.nnz)
        rc = _lib.load().sblas_csc_bind_values(self.m, self.n, self.nnz, _ptr(val),
                                               _ptr(self.work), self.work_bytes,
                                               _stream_ptr(self.device))
        _lib.check(rc)
        self.bound = True

    def __call__(self, val: torch.Tensor | None, x: torch.Tensor, y: torch.Tensor,
                 alpha: float = 1.0, beta: float = 0.0) -> torch.Tensor:
        if val is None and not getattr(self, "bound", False):
            raise ValueError("no values: pass val or bind() them first")
        if _require_cuda(val, x, y) != self.device:
            raise ValueError("val, x and y must be on the plan's device")
        for what, t in (("val", val), ("x", x), ("y", y)):
            _require_dtype(what, t, torch.float64)
        _require_len("val", val, self.nnz)
        _require_len("x", x, self.n)
        if y.numel() != self.m:
            raise ValueError("y must have m entries")
        rc = _lib.load().sblas_dcscmv_analysed(self.m, self.n, self.nnz, float(alpha), _ptr(val),
                                               _ptr(x), float(beta), _ptr(y), _ptr(self.work),
                                               self.work_bytes, _stream_ptr(self.device))
        _lib.check(rc)
        return y


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
        _require_dtype("rowptr", rowptr, torch.int32)
        _require_dtype("col", col, torch.int32)
        _require_len("val", val, col.numel())
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
        if _require_cuda(x, y) != self.device:
            raise ValueError("x and y must be on the plan's device")
        _require_dtype("x", x, torch.float64)
        _require_dtype("y", y, torch.float64)
        n = self.n if self.n is not None else x.numel()
        if y.numel() != self.m or x.numel() < n:
            raise ValueError("shape mismatch")
        lib = _lib.load()
        rc = lib.sblas_dcsrmv_analysed(self.kernel, self.m, n, self.nnz, float(alpha),
                                       _ptr(self.val), self.vk, _ptr(self.rowptr), _ptr(self.col),
                                       _ptr(x), float(beta), _ptr(y), self.sigma, _ptr(self.work),
                                       self.work_bytes, _stream_ptr(self.device))
        _lib.check(rc)
        return y


def _val_kind(val: torch.Tensor | None) -> int:
    if val is None:
        return VAL_PATTERN
    if val.dtype == torch.float64:
        return VAL_F64
    if val.dtype == torch.float32:
        return VAL_F32
    raise TypeError("val must be float64, float32 or None")


def batch_default_s(k: int) -> int:
    return int(_lib.load().sblas_batch_default_s(k))


class BatchPlan:
    """Many CSR matrices, k right-hand sides each: Y_i = alpha*A_i*X_i + beta*Y_i.

    matrices: list of (rowptr, col, val) with int32 indices and val float64,
    float32 or None (pattern; every matrix of a batch has the same value
    kind), or (rowptr, col, val, row_ids[, val_perm]): stored row r is row
    row_ids[r] of Y (int32, ascending; None: r) and unlisted rows of Y are
    left untouched; stored entry p has value val[val_perm[p]] (int32; None:
    val[p]).  xs[i]: float64 (n_i, k) row-major (or (n_i,) for k = 1);
    ys[i]: float64 (m_i, k).  The plan (sblas_batch_plan_create) copies the
    descriptors to the device and partitions all matrices into units of
    32*s nonzeros; each call is one persistent kernel plus the carry fix-up
    (sblas_batch_spmm): no allocation, no copy, graph-capturable.  s = 0
    takes the library default for k (see tune.batch_s for a measured pick).
    """

    def __init__(self, matrices, xs, ys, k: int, alpha: float = 1.0, beta: float = 0.0,
                 s: int = 0):
        if not (len(matrices) == len(xs) == len(ys)) or not matrices:
            raise ValueError("need one x and one y per matrix")
        flat = [t for mat in matrices for t in mat] + list(xs) + list(ys)
        dev = _require_cuda(*flat)
        matrices = [tuple(mat) + (None,) * (5 - len(mat)) for mat in matrices]
        kinds = {_val_kind(mat[2]) for mat in matrices}
        if len(kinds) != 1:
            raise TypeError("all matrices of a batch have the same value kind")
        self.vk = kinds.pop()
        self.k = int(k)
        self.device = dev
        self.matrices, self.xs, self.ys = list(matrices), list(xs), list(ys)
        arr = (_lib.BatchMatrix * len(matrices))()
        for i, ((rp, col, val, rid, vperm), x, y) in enumerate(zip(matrices, xs, ys)):
            if rp.dtype != torch.int32 or col.dtype != torch.int32:
                raise TypeError("rowptr and col must be int32")
            if x.dtype != torch.float64 or y.dtype != torch.float64:
                raise TypeError("x and y must be float64")
            m = rp.numel() - 1
            n = x.shape[0]
            if rid is not None and (rid.dtype != torch.int32 or rid.numel() != m):
                raise ValueError(f"matrix {i}: row_ids must be int32 with one entry per row")
            if vperm is not None and (vperm.dtype != torch.int32 or vperm.numel() != col.numel()):
                raise ValueError(f"matrix {i}: val_perm must be int32 with one entry per nonzero")
            if vperm is None:
                _require_len(f"matrix {i}: val", val, col.numel())
            if (y.shape[0] != m if rid is None else y.shape[0] < m) or \
                    (x.dim() > 1 and x.shape[1] != self.k) or \
                    (y.dim() > 1 and y.shape[1] != self.k) or (self.k > 1 and x.dim() != 2):
                raise ValueError(f"matrix {i}: x must be (n, k) and y (m, k)")
            arr[i] = _lib.BatchMatrix(m, n, col.numel(), _ptr(val).value, _ptr(rp).value,
                                      _ptr(col).value, _ptr(x).value, self.k, _ptr(y).value,
                                      self.k, float(alpha), float(beta), _ptr(rid).value,
                                      _ptr(vperm).value)
        lib = _lib.load()
        h = C.c_void_p()
        with torch.cuda.device(dev):
            rc = lib.sblas_batch_plan_create(len(matrices), arr, self.k, self.vk, int(s),
                                             _stream_ptr(dev), C.byref(h))
        _lib.check(rc)
        self._h = h
        units, s_out, nbytes = C.c_longlong(), C.c_int(), C.c_size_t()
        _lib.check(lib.sblas_batch_plan_info(h, C.byref(units), C.byref(s_out), C.byref(nbytes)))
        self.units, self.s, self.device_bytes = units.value, s_out.value, nbytes.value

    def __call__(self) -> None:
        rc = _lib.load().sblas_batch_spmm(self._h, _stream_ptr(self.device))
        _lib.check(rc)

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().sblas_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SpmmPlan(BatchPlan):
    """One CSR matrix with k right-hand sides, X, Y, alpha and beta given per
    call: Y = alpha*A*X + beta*Y (sblas_batch_spmm_xy).  The structure is
    fixed at construction; the values may be replaced per call (val=, same
    dtype as at construction).

    split16=True runs a k = 16 product as two k = 8 passes over the column
    halves of X and Y (row stride 16).  The default is the single k = 16
    pass: its lanes-over-columns kernel reads each row of X once (128
    bytes) and measured 0.76 ms against 0.95 ms for the two passes on a
    1M-row power-law matrix with 20.1M nonzeros."""

    def __init__(self, rowptr: torch.Tensor, col: torch.Tensor, val: torch.Tensor | None,
                 n: int, k: int, s: int = 0, row_ids: torch.Tensor | None = None,
                 m_out: int | None = None, val_perm: torch.Tensor | None = None,
                 split16: bool = False):
        dev = _require_cuda(rowptr, col, val, row_ids, val_perm)
        m = rowptr.numel() - 1 if m_out is None else int(m_out)
        # placeholders fixing the shapes; every call passes its own X and Y
        xs = torch.empty((max(n, 1), k), dtype=torch.float64, device=dev)
        ys = torch.empty((max(m, 1), k), dtype=torch.float64, device=dev)
        super().__init__([(rowptr, col, val, row_ids, val_perm)], [xs[:n]], [ys[:m]], k, s=s)
        self.m, self.n = m, n
        self.val_dtype = None if val is None else val.dtype
        self._half = None
        if k == 16 and split16:
            self._half = SpmmPlan(rowptr, col, val, n, 8, s=s, row_ids=row_ids, m_out=m_out,
                                  val_perm=val_perm)

    def close(self) -> None:
        if getattr(self, "_half", None) is not None:
            self._half.close()
            self._half = None
        super().close()

    def _check_val(self, val):
        if val is None:
            return
        _require_cuda(val)
        if self.val_dtype is None or val.dtype != self.val_dtype:
            raise TypeError("values must have the dtype the plan was built with")
        if val.numel() != self.matrices[0][1].numel():
            raise ValueError("one value per stored entry")

    def __call__(self, x: torch.Tensor, y: torch.Tensor, alpha: float = 1.0, beta: float = 0.0,
                 val: torch.Tensor | None = None) -> torch.Tensor:
        _require_cuda(x, y)
        self._check_val(val)
        if x.dtype != torch.float64 or y.dtype != torch.float64:
            raise TypeError("x and y must be float64")
        if x.shape[0] != self.n or y.shape[0] != self.m or x.numel() != self.n * self.k or \
                y.numel() != self.m * self.k:
            raise ValueError("x must be (n, k) and y (m, k)")
        if _require_cuda(x, y) != self.device:
            raise ValueError("x and y must be on the plan's device")
        lib = _lib.load()
        if self._half is not None and x.is_contiguous() and y.is_contiguous():
            # two k = 8 passes: columns 0-7, then 8-15 (64 bytes on, row stride 16)
            for off in (0, 64):
                rc = lib.sblas_batch_spmm_xy(self._half._h, _ptr(val),
                                             C.c_void_p(x.data_ptr() + off), 16,
                                             C.c_void_p(y.data_ptr() + off), 16, float(alpha),
                                             float(beta), _stream_ptr(self.device))
                _lib.check(rc)
            return y
        rc = lib.sblas_batch_spmm_xy(self._h, _ptr(val), _ptr(x), self.k, _ptr(y), self.k,
                                     float(alpha), float(beta), _stream_ptr(self.device))
        _lib.check(rc)
        return y

    def sddmm(self, g: torch.Tensor, x: torch.Tensor, dval: torch.Tensor) -> torch.Tensor:
        """dval[p] = G[row(p), :] . X[col(p), :] (the values' adjoint)."""
        _require_cuda(g, x, dval)
        if g.dtype != torch.float64 or x.dtype != torch.float64:
            raise TypeError("g and x must be float64")
        if g.shape[0] != self.m or x.shape[0] != self.n or dval.dtype != self.val_dtype or \
                g.numel() != self.m * self.k or x.numel() != self.n * self.k or \
                dval.numel() != self.matrices[0][1].numel():
            raise ValueError("g must be (m, k), x (n, k), dval one value per stored entry "
                             "of the values' dtype")
        rc = _lib.load().sblas_batch_sddmm(self._h, _ptr(g), self.k, _ptr(x), self.k, _ptr(dval),
                                           _stream_ptr(self.device))
        _lib.check(rc)
        return dval


def zero_(t: torch.Tensor) -> torch.Tensor:
    """t[:] = 0 on the device (cudaMemsetAsync on the current stream)."""
    dev = _require_cuda(t)
    rc = _lib.load().sblas_zero(_ptr(t), t.numel() * t.element_size(), _stream_ptr(dev))
    _lib.check(rc)
    return t


def csr_transpose(m: int, n: int, rowptr: torch.Tensor,
                  col: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Device CSR structure of A^T: (t_rowptr, t_col, perm) with the values of
    A^T equal to val[perm]."""
    dev = _require_cuda(rowptr, col)
    _require_dtype("rowptr", rowptr, torch.int32)
    _require_dtype("col", col, torch.int32)
    _require_len("rowptr", rowptr, m + 1)
    nnz = col.numel()
    lib = _lib.load()
    wb = int(lib.sblas_csr_transpose_workspace_bytes(m, n, nnz))
    work = torch.empty(max(wb, 1), dtype=torch.uint8, device=dev)
    t_rowptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
    t_col = torch.empty(nnz, dtype=torch.int32, device=dev)
    perm = torch.empty(nnz, dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        rc = lib.sblas_csr_transpose(m, n, nnz, _ptr(rowptr), _ptr(col), _ptr(t_rowptr),
                                     _ptr(t_col), _ptr(perm), _ptr(work), wb, _stream_ptr(dev))
    _lib.check(rc)
    return t_rowptr, t_col, perm


def gather_values(val: torch.Tensor, perm: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
    """out[p] = val[perm[p]] on the device (FP64 or FP32 values)."""
    dev = _require_cuda(val, perm, out)
    _require_dtype("perm", perm, torch.int32)
    _require_dtype("out", out, val.dtype)
    _require_len("out", out, perm.numel())
    rc = _lib.load().sblas_gather_values(perm.numel(), _val_kind(val), _ptr(val), _ptr(perm),
                                         _ptr(out), _stream_ptr(dev))
    _lib.check(rc)
    return out


def csr_filter_x(rowptr: torch.Tensor, col: torch.Tensor, val: torch.Tensor | None,
                 x: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor | None]:
    """spMspV's x-zero filter on the device (src/dspmv_mgpu_v1.cu:29-40): the
    CSR matrix of the nonzeros whose x[col] != 0, in storage order.  Reads the
    kept count back (one synchronisation) to size the outputs."""
    dev = _require_cuda(rowptr, col, val, x)
    if val is not None and val.dtype != torch.float64:
        raise TypeError("val must be float64 or None")
    _require_dtype("rowptr", rowptr, torch.int32)
    _require_dtype("col", col, torch.int32)
    _require_dtype("x", x, torch.float64)
    m = rowptr.numel() - 1
    nnz = col.numel()
    _require_len("val", val, nnz)
    lib = _lib.load()
    wb = int(lib.sblas_csr_filter_x_workspace_bytes(nnz))
    work = torch.empty(max(wb, 1), dtype=torch.uint8, device=dev)
    orp = torch.empty(m + 1, dtype=torch.int32, device=dev)
    ocol = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    oval = None if val is None else torch.empty(max(nnz, 1), dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        rc = lib.sblas_csr_filter_x(m, nnz, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(x),
                                    _ptr(orp), _ptr(ocol), _ptr(oval), _ptr(work), wb,
                                    _stream_ptr(dev))
    _lib.check(rc)
    k = int(orp[m].item())
    return orp, ocol[:k], (None if oval is None else oval[:k])


def spmspv(rowptr: torch.Tensor, col: torch.Tensor, val: torch.Tensor | None, x: torch.Tensor,
           y: torch.Tensor, alpha: float = 1.0, beta: float = 0.0,
           kernel: int = KERNEL_MERGEPATH) -> torch.Tensor:
    """y = alpha*A'*x + beta*y with A' = A without the nonzeros whose x entry
    is zero, as spMspV_mgpu_v1 computes it (src/dspmv_mgpu_v1.cu:19-74), on
    device arrays: the filter and the product both run on the GPU."""
    orp, ocol, oval = csr_filter_x(rowptr, col, val, x)
    return csrmv(orp, ocol, oval, x, y, alpha, beta, n=x.numel(), kernel=kernel)


def check_device(device: torch.device | None = None, clear: bool = True) -> None:
    """Waits for the current stream of `device`, then raises SblasError
    (SBLAS_ERR_TIMEOUT) if a tile kernel launched on that device gave up one
    of its bounded waits since the last check: the y of that launch is only
    partly written.  clear=True resets the device's sticky word."""
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    with torch.cuda.device(dev):
        rc = _lib.load().sblas_stream_status(_stream_ptr(dev), 1 if clear else 0)
    _lib.check(rc)
