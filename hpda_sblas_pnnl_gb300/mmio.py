"""MatrixMarket files into the library's formats (include/mmio.h).

The reference's drivers read a coordinate file entry by entry with fscanf
(test/dspmv_test_dgx1.cu:133-181), sort it by row (sortCOORow) and convert
it to CSR (coo2csr).  Here the file is parsed by the library's
multi-threaded reader (sblas_mm_read_coo) and converted by the library's
coo2csr (a device sort).  Arrays are numpy: int32 indices, float64 values,
0-based.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._lib import MMHeader, SblasError, load


def _path(path) -> bytes:
    return os.fsencode(os.fspath(path))


def _raise(lib) -> None:
    raise SblasError(lib.sblas_last_status(), lib.sblas_last_error().decode())


def read_header(path) -> dict:
    """{'m', 'n', 'nnz', 'typecode'} of a coordinate file."""
    lib = load()
    h = MMHeader()
    if lib.sblas_mm_read_header(_path(path), C.byref(h)) != 0:
        _raise(lib)
    return {"m": h.m, "n": h.n, "nnz": h.nnz, "typecode": h.typecode.decode()}


def read_coo(path, expand_symmetric: bool = False, threads: int = 0):
    """(m, n, row, col, val) in file order.  expand_symmetric mirrors the
    off-diagonal entries of symmetric / skew-symmetric files (the reference
    keeps the stored triangle only)."""
    lib = load()
    h = read_header(path)
    need = C.c_longlong(0)
    mirror = expand_symmetric and h["typecode"][3] != "G"
    cap = 2 * h["nnz"] if mirror else h["nnz"]   # at most one mirror per entry
    row = np.empty(cap, np.int32)
    col = np.empty(cap, np.int32)
    val = np.empty(cap, np.float64)
    if cap == 0:
        return h["m"], h["n"], row, col, val
    rc = lib.sblas_mm_read_coo(_path(path), int(bool(expand_symmetric)), int(threads), cap,
                               row.ctypes.data, col.ctypes.data, val.ctypes.data,
                               C.byref(need))
    if rc != 0:
        _raise(lib)
    k = need.value
    if k < cap:
        row, col, val = row[:k].copy(), col[:k].copy(), val[:k].copy()
    return h["m"], h["n"], row, col, val


def read_csr(path, expand_symmetric: bool = False, threads: int = 0):
    """(m, n, rowptr, col, val): read_coo, then the library's coo2csr
    (stable by row: entries of a row keep their file order)."""
    from . import api
    m, n, row, col, val = read_coo(path, expand_symmetric, threads)
    v, p, c = api.coo2csr(m, n, int(row.size), val, row, col)
    return m, n, p, c, v


__all__ = ["read_header", "read_coo", "read_csr"]
