"""ctypes loader of the oracle (oracle/liboracle.so) and of the reference's
own CPU functions compiled from its sources (oracle/_ref/libref_cpu.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_cpu.so"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_o: C.CDLL | None = None
_r: C.CDLL | None = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def _lib() -> C.CDLL:
    global _o
    if _o is None:
        if not LIB.exists():
            build()
        _o = C.CDLL(str(LIB))
        spmv_args = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp, _dp]
        for name in ("oracle_csr_spmv", "oracle_coo_spmv", "oracle_csc_spmv",
                     "oracle_csr_spmv_dot2"):
            getattr(_o, name).argtypes = spmv_args
            getattr(_o, name).restype = None
        _o.oracle_csr_spmv_omp.argtypes = spmv_args + [C.c_int]
        _o.oracle_csr_spmv_nnz_split.argtypes = spmv_args + [C.c_int]
        _o.oracle_csr_spmv_nnz_split.restype = C.c_int
        _o.oracle_nnz_partition.argtypes = [C.c_int, C.c_int, _ip, C.c_int, _ip]
        _o.oracle_nnz_partition.restype = C.c_int
        _o.oracle_get_row_from_index.argtypes = [C.c_int, _ip, C.c_int]
        _o.oracle_find_first_in_sorted.argtypes = [_ip, C.c_int, C.c_int]
        _o.oracle_find_last_in_sorted.argtypes = [_ip, C.c_int, C.c_int]
        _o.oracle_gen_g.argtypes = [C.c_int, _ip, _ip, _dp]
        _o.oracle_gen_g.restype = C.c_longlong
        for name in ("oracle_coo2csr", "oracle_coo2csc"):
            getattr(_o, name).argtypes = [C.c_int, C.c_int, C.c_int, _dp, _ip, _ip, _dp, _ip, _ip]
        _o.oracle_csr_spmm.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp,
                                       C.c_int, _dp, _dp, C.c_int, C.c_int]
        _o.oracle_csr_spmm_t.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _ip, _ip, _dp, C.c_int,
                                         _dp, C.c_int]
        _o.oracle_csr_sddmm.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, C.c_int, _dp, C.c_int,
                                        _dp]
        _o.oracle_csr_filter_x.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _ip, _ip, _dp]
        _o.oracle_csr_filter_x.restype = C.c_longlong
        _o.oracle_mm_read_fscanf.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                             C.POINTER(C.c_longlong), C.POINTER(C.c_int), _ip,
                                             _ip, _dp]
        _o.oracle_mm_read_fscanf.restype = C.c_int
    return _o


def ref_available() -> bool:
    return REF_LIB.exists()


def _ref() -> C.CDLL:
    global _r
    if _r is None:
        if not REF_LIB.exists():
            raise FileNotFoundError(f"{REF_LIB} not built (oracle/ref_build.sh)")
        _r = C.CDLL(str(REF_LIB))
        spmv_args = [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp, _dp]
        _r.ref_csr_spmv_cpu.argtypes = spmv_args
        _r.ref_coo_spmv_cpu.argtypes = spmv_args
        _r.ref_csr_spmv_cpu_threads.argtypes = spmv_args + [C.c_int]
        _r.ref_get_row_from_index.argtypes = [C.c_int, _ip, C.c_int]
        _r.ref_find_first_in_sorted.argtypes = [_ip, C.c_int, C.c_int]
        _r.ref_find_last_in_sorted.argtypes = [_ip, C.c_int, C.c_int]
    return _r


def _d(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _i(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def _ab(alpha, beta):
    return C.byref(C.c_double(alpha)), C.byref(C.c_double(beta))


def csr_spmv(m, n, rowptr, col, val, x, y, alpha=1.0, beta=0.0, threads=0, dot2=False):
    """Returns a new y (input y untouched)."""
    y = np.array(y, dtype=np.float64, copy=True)
    a, b = _ab(alpha, beta)
    args = (m, n, int(col.size), a, _d(val), _i(rowptr), _i(col), _d(x), b, _d(y))
    if dot2:
        _lib().oracle_csr_spmv_dot2(*args)
    elif threads:
        _lib().oracle_csr_spmv_omp(*args, threads)
    else:
        _lib().oracle_csr_spmv(*args)
    return y


def _dn(a):
    return None if a is None else _d(a)


def _k2(a, rows):
    """(rows, k) C-contiguous float64 view of a 1-D or 2-D array, and k."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.ndim == 1:
        a = a.reshape(rows, 1)
    return a, a.shape[1]


def csr_spmm(m, n, rowptr, col, val, x, y, alpha=1.0, beta=0.0, threads=0):
    """Y = alpha*A*X + beta*Y for row-major X (n, k), Y (m, k); val None:
    pattern.  Returns a new Y (input untouched), shaped like y."""
    shape = np.shape(y)
    x, k = _k2(x, n)
    y = np.array(_k2(y, m)[0], copy=True)
    a, b = _ab(alpha, beta)
    _lib().oracle_csr_spmm(m, n, k, a, _dn(val), _i(rowptr), _i(col), _d(x), k, b, _d(y), k,
                           threads)
    return y.reshape(shape)


def csr_spmm_t(m, n, rowptr, col, val, g):
    """dX = A^T G for G (m, k); returns (n, k) (or (n,) for 1-D g)."""
    g1 = np.ndim(g) == 1
    g, k = _k2(g, m)
    dx = np.zeros((n, k))
    _lib().oracle_csr_spmm_t(m, n, k, _dn(val), _i(rowptr), _i(col), _d(g), k, _d(dx), k)
    return dx[:, 0] if g1 else dx


def csr_sddmm(m, n, rowptr, col, g, x):
    """dval[p] = sum_c G[row(p), c] * X[col(p), c]."""
    g, k = _k2(g, m)
    x, _ = _k2(x, n)
    dval = np.zeros(col.size)
    _lib().oracle_csr_sddmm(m, k, _i(rowptr), _i(col), _d(g), k, _d(x), k, _d(dval))
    return dval


def coo_spmv(m, n, row, col, val, x, y, alpha=1.0, beta=0.0):
    y = np.array(y, dtype=np.float64, copy=True)
    a, b = _ab(alpha, beta)
    _lib().oracle_coo_spmv(m, n, int(col.size), a, _d(val), _i(row), _i(col), _d(x), b, _d(y))
    return y


def csc_spmv(m, n, colptr, row, val, x, y, alpha=1.0, beta=0.0):
    y = np.array(y, dtype=np.float64, copy=True)
    a, b = _ab(alpha, beta)
    _lib().oracle_csc_spmv(m, n, int(row.size), a, _d(val), _i(colptr), _i(row), _d(x), b, _d(y))
    return y


def csr_spmv_nnz_split(m, n, rowptr, col, val, x, y, nparts, alpha=1.0, beta=0.0):
    y = np.array(y, dtype=np.float64, copy=True)
    a, b = _ab(alpha, beta)
    rc = _lib().oracle_csr_spmv_nnz_split(m, n, int(col.size), a, _d(val), _i(rowptr), _i(col),
                                          _d(x), b, _d(y), nparts)
    if rc != 0:
        raise ValueError("nnz < nparts")
    return y


def nnz_partition(m, rowptr, nparts):
    """The reference's v1 split (src/dspmv_mgpu_v1.cu:120-152): an
    (nparts, 7) int array of start_idx, end_idx, start_row, end_row,
    start_flag, end_flag, rows per part."""
    nnz = int(rowptr[m]) if m > 0 else 0
    out = np.zeros((max(nparts, 1), 7), np.int32)
    if _lib().oracle_nnz_partition(m, nnz, _i(rowptr), nparts, _i(out)) != 0:
        raise ValueError("nnz < nparts")
    return out


def get_row_from_index(n, a, idx):
    return _lib().oracle_get_row_from_index(n, _i(a), idx)


def find_first_in_sorted(a, n, key):
    return _lib().oracle_find_first_in_sorted(_i(a), n, key)


def find_last_in_sorted(a, n, key):
    return _lib().oracle_find_last_in_sorted(_i(a), n, key)


def gen_g(n):
    """The reference's 'g' matrix as row-major COO (row, col, val)."""
    nnz = _lib().oracle_gen_g(n, None, None, None)
    if nnz < 0:
        raise ValueError("n must be a positive multiple of 8")
    r = np.empty(nnz, np.int32)
    c = np.empty(nnz, np.int32)
    v = np.empty(nnz, np.float64)
    _lib().oracle_gen_g(n, _i(r), _i(c), _d(v))
    return r, c, v


def coo2csr(m, n, val, row, col):
    nnz = int(row.size)
    v = np.empty(nnz, np.float64)
    p = np.empty(m + 1, np.int32)
    c = np.empty(nnz, np.int32)
    _lib().oracle_coo2csr(m, n, nnz, _d(val), _i(row), _i(col), _d(v), _i(p), _i(c))
    return v, p, c


def csr_filter_x(m, rowptr, col, val, x):
    """(rowptr, col, val) of the nonzeros whose x[col] != 0 (spMspV's filter)."""
    nnz = int(col.size)
    orp = np.empty(m + 1, np.int32)
    oc = np.empty(max(nnz, 1), np.int32)
    ov = np.empty(max(nnz, 1), np.float64)
    k = _lib().oracle_csr_filter_x(m, _i(rowptr), _i(col), _d(val), _d(x), _i(orp), _i(oc),
                                   _d(ov))
    return orp, oc[:k].copy(), ov[:k].copy()


def mm_read_fscanf(path):
    """The reference's per-entry fscanf reading of a coordinate file
    (test/dspmv_test_dgx1.cu:133-181) -> (m, n, row, col, val), 0-based.
    Raises ValueError where that loop cannot read the file."""
    lib = _lib()
    p = os.fsencode(str(path))
    m, n, kind, nnz = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
    args = (C.byref(m), C.byref(n), C.byref(nnz), C.byref(kind))
    if lib.oracle_mm_read_fscanf(p, *args, None, None, None) != 0:
        raise ValueError(f"{path}: unreadable MatrixMarket header")
    row = np.empty(nnz.value, np.int32)
    col = np.empty(nnz.value, np.int32)
    val = np.empty(nnz.value, np.float64)
    if lib.oracle_mm_read_fscanf(p, *args, _i(row), _i(col), _d(val)) != 0:
        raise ValueError(f"{path}: an entry fscanf cannot read")
    return m.value, n.value, row, col, val


def coo2csc(m, n, val, row, col):
    nnz = int(row.size)
    v = np.empty(nnz, np.float64)
    p = np.empty(n + 1, np.int32)
    r = np.empty(nnz, np.int32)
    _lib().oracle_coo2csc(m, n, nnz, _d(val), _i(row), _i(col), _d(v), _i(p), _i(r))
    return v, p, r


# ---- the reference's own CPU functions (compiled from its sources) --------

def ref_csr_spmv(m, n, rowptr, col, val, x, y, alpha=1.0, beta=0.0, threads=0):
    y = np.array(y, dtype=np.float64, copy=True)
    a, b = _ab(alpha, beta)
    args = (m, n, int(col.size), a, _d(val), _i(rowptr), _i(col), _d(x), b, _d(y))
    if threads:
        _ref().ref_csr_spmv_cpu_threads(*args, threads)
    else:
        _ref().ref_csr_spmv_cpu(*args)
    return y


def ref_coo_spmv(m, n, row, col, val, x, y, alpha=1.0, beta=0.0):
    y = np.array(y, dtype=np.float64, copy=True)
    a, b = _ab(alpha, beta)
    _ref().ref_coo_spmv_cpu(m, n, int(col.size), a, _d(val), _i(row), _i(col), _d(x), b, _d(y))
    return y


def ref_get_row_from_index(n, a, idx):
    return _ref().ref_get_row_from_index(n, _i(a), idx)


def ref_find_first_in_sorted(a, n, key):
    return _ref().ref_find_first_in_sorted(_i(a), n, key)


def ref_find_last_in_sorted(a, n, key):
    return _ref().ref_find_last_in_sorted(_i(a), n, key)
