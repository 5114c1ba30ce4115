"""The reference's multi-GPU nnz split, one process per device.

spMV_mgpu_v1 (src/dspmv_mgpu_v1.cu:76-360) cuts A's nonzeros into ngpu equal
ranges, runs every range on its own GPU and merges the row ranges back into
y on the host, fixing the rows a cut splits.  Here every rank of a
torch.distributed process group is one part: the cut points, the parts' row
pointers and the merge are the library's (sblas_nnz_partition,
sblas_part_rowptr, sblas_merge_parts: the reference's arithmetic, 64-bit
cut points), the per-part SpMV is this rank's device kernel, and the
exchange is one all_gather of the parts' row ranges (x is replicated; the
only data crossing ranks is y).  Given the same per-part results the merged
rows equal the reference's bit for bit; the empty rows outside every part,
which the reference leaves untouched, get beta*y0 unless the library's
reference-compatibility mode is on.

`compute` replaces the per-part product (the tests run the ranks on CPU
with the gloo backend and the oracle's row loop as the product); by default
it is the tile kernel on the rank's current CUDA device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def partition(rowptr: np.ndarray, nparts: int) -> list[_lib.NnzPart]:
    """The v1 cut of the CSR row pointer (int32, m + 1 entries) into nparts."""
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    m = rowptr.size - 1
    parts = (_lib.NnzPart * max(nparts, 1))()
    rc = _lib.load().sblas_nnz_partition(m, int(rowptr[-1]) if m >= 0 else 0, _ip(rowptr),
                                         int(nparts), C.cast(parts, C.c_void_p))
    _lib.check(rc)
    return list(parts)


def part_rowptr(rowptr: np.ndarray, part: _lib.NnzPart) -> np.ndarray:
    """Row pointer of one part (part.m + 1 entries, rebased, rows clipped)."""
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    out = np.empty(part.m + 1, np.int32)
    _lib.check(_lib.load().sblas_part_rowptr(_ip(rowptr), C.byref(part), _ip(out)))
    return out


def merge(parts: list[_lib.NnzPart], pieces: list[np.ndarray], beta: float,
          y: np.ndarray) -> np.ndarray:
    """y (holding y0) <- the parts' row ranges, merged in the reference's
    order (src/dspmv_mgpu_v1.cu:304-319)."""
    if len(pieces) != len(parts):
        raise ValueError("one piece per part")
    pieces = [np.ascontiguousarray(p, dtype=np.float64) for p in pieces]
    for p, piece in zip(parts, pieces):
        if piece.size < p.m:
            raise ValueError("a piece holds fewer rows than its part")
    if y.dtype != np.float64 or not y.flags.c_contiguous:
        raise TypeError("y must be a C-contiguous float64 array")
    arr = (_lib.NnzPart * len(parts))(*parts)
    ptrs = (C.c_void_p * len(pieces))(*[p.ctypes.data for p in pieces])
    rc = _lib.load().sblas_merge_parts(len(parts), C.cast(arr, C.c_void_p),
                                       C.cast(ptrs, C.c_void_p), float(beta),
                                       y.ctypes.data_as(C.POINTER(C.c_double)))
    _lib.check(rc)
    return y


def _device_product(prow, pcol, pval, x, py0, alpha, beta):
    """This rank's part on its current CUDA device (the tile kernel)."""
    import torch

    from . import ops
    dev = torch.device("cuda", torch.cuda.current_device())
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)   # noqa: E731
    y = t(py0)
    ops.csrmv(t(prow), t(pcol), t(pval), t(x), y, alpha, beta)
    return y.cpu().numpy()


def dist_csrmv(m: int, n: int, rowptr: np.ndarray, col: np.ndarray, val: np.ndarray,
               x: np.ndarray, y: np.ndarray, alpha: float = 1.0, beta: float = 0.0,
               group=None, compute=None) -> np.ndarray:
    """y = alpha*A*x + beta*y over the ranks of `group` (every rank passes the
    same host arrays; every rank returns the whole merged y, in place)."""
    import torch
    import torch.distributed as dist

    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    parts = partition(rowptr[: m + 1], world)
    p = parts[rank]
    prow = part_rowptr(rowptr, p)
    lo, hi = p.start_idx, p.end_idx + 1
    py0 = np.array(y[p.start_row: p.end_row + 1], dtype=np.float64)
    fn = compute or _device_product
    piece = np.asarray(fn(prow, col[lo:hi], val[lo:hi], x, py0, alpha, beta), dtype=np.float64)
    # exchange: the parts' row ranges, padded to the longest
    width = max(q.m for q in parts)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else "cpu"
    buf = torch.zeros(width, dtype=torch.float64, device=dev)
    buf[: p.m] = torch.from_numpy(piece[: p.m]).to(dev)
    got = [torch.empty(width, dtype=torch.float64, device=dev) for _ in range(world)]
    dist.all_gather(got, buf, group=group)
    pieces = [g.cpu().numpy()[: q.m] for g, q in zip(got, parts)]
    merge(parts, pieces, beta, y)
    # rows before the first and after the last nonzero belong to no part: the
    # reference leaves them untouched (src/dspmv_mgpu_v1.cu:132-157); here,
    # as everywhere outside reference-compatibility mode, they get beta*y0
    if not _lib.load().sblas_get_compat_mode():
        for sl in (slice(0, parts[0].start_row), slice(parts[-1].end_row + 1, m)):
            y[sl] = 0.0 if beta == 0.0 else beta * y[sl]
    return y


__all__ = ["partition", "part_rowptr", "merge", "dist_csrmv"]
