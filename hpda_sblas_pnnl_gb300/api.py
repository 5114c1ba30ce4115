"""Python mirror of the reference's entry points (include/spmv_kernel.h).

Same names, argument order and meaning as the C functions the reference's
drivers call (test/dspmv_test_smt.cu:460-511): host arrays in, y updated in
place, an spmv_ret of per-phase seconds out.  Arrays are numpy (float64 and
int32, C-contiguous); alpha and beta are Python floats (the C ABI takes
pointers to them).  A failed call raises SblasError with the library's
message, where the reference would exit the process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import SblasError, SpmvRet, load

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _d(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_dp)


def _i(a: np.ndarray | None):
    if a is None:
        return None
    if a.dtype != np.int32 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous int32 array")
    return a.ctypes.data_as(_ip)


SBLAS_ERR_ARG = -1


def _lengths(*arrays) -> None:
    """(name, array, length) triples: raises SblasError(SBLAS_ERR_ARG) when an
    array holds fewer elements than its size arguments say.  The C entry
    points take bare pointers and would read past its end.  Lengths of zero
    or less are left to the library, which rejects negative sizes itself."""
    for name, a, need in arrays:
        if a is not None and need > 0 and np.asarray(a).size < need:
            raise SblasError(SBLAS_ERR_ARG,
                             f"{name} holds {np.asarray(a).size} elements, {need} needed")


def _csr_lengths(m, n, nnz, val, rowptr, col, x, y) -> None:
    _lengths(("csrVal", val, nnz), ("csrRowPtr", rowptr, m + 1), ("csrColIndex", col, nnz),
             ("x", x, n), ("y", y, m))


def _csc_lengths(m, n, nnz, val, colptr, rowidx, x, y) -> None:
    _lengths(("cscVal", val, nnz), ("cscColPtr", colptr, n + 1), ("cscRowIdx", rowidx, nnz),
             ("x", x, n), ("y", y, m))


def _coo_lengths(m, n, nnz, val, row, col, x=None, y=None) -> None:
    _lengths(("cooVal", val, nnz), ("cooRowIdx", row, nnz), ("cooColIdx", col, nnz),
             ("x", x, n), ("y", y, m))


def _scalar(v: float):
    return C.byref(C.c_double(float(v)))


def _done(r: SpmvRet) -> SpmvRet:
    if r.failed():
        lib = load()
        raise SblasError(lib.sblas_last_status(), lib.sblas_last_error().decode())
    return r


def set_compat_mode(mode: int) -> None:
    """1 = reproduce the reference's ngpu=1 quirks (see include/sblas_gb300.h)."""
    load().sblas_set_compat_mode(int(mode))


def spMV_mgpu_baseline(m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta, y, ngpu=1):
    _csr_lengths(m, n, nnz, csrVal, csrRowPtr, csrColIndex, x, y)
    return _done(load().spMV_mgpu_baseline(m, n, nnz, _scalar(alpha), _d(csrVal), _i(csrRowPtr),
                                           _i(csrColIndex), _d(x), _scalar(beta), _d(y), ngpu))


def spMV_mgpu_baseline_csc(m, n, nnz, alpha, cscVal, cscColPtr, cscRowIdx, x, beta, y, ngpu=1):
    _csc_lengths(m, n, nnz, cscVal, cscColPtr, cscRowIdx, x, y)
    return _done(load().spMV_mgpu_baseline_csc(m, n, nnz, _scalar(alpha), _d(cscVal),
                                               _i(cscColPtr), _i(cscRowIdx), _d(x),
                                               _scalar(beta), _d(y), ngpu))


def spMV_mgpu_baseline_coo(m, n, nnz, alpha, cooVal, cooRowIdx, cooColIdx, x, beta, y, ngpu=1):
    _coo_lengths(m, n, nnz, cooVal, cooRowIdx, cooColIdx, x, y)
    return _done(load().spMV_mgpu_baseline_coo(m, n, nnz, _scalar(alpha), _d(cooVal),
                                               _i(cooRowIdx), _i(cooColIdx), _d(x),
                                               _scalar(beta), _d(y), ngpu))


def spMV_mgpu_v1(m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta, y, ngpu=1, kernel=2):
    _csr_lengths(m, n, nnz, csrVal, csrRowPtr, csrColIndex, x, y)
    return _done(load().spMV_mgpu_v1(m, n, nnz, _scalar(alpha), _d(csrVal), _i(csrRowPtr),
                                     _i(csrColIndex), _d(x), _scalar(beta), _d(y), ngpu, kernel))


def spMV_mgpu_v1_numa(m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta, y, ngpu=1,
                      kernel=1, numa_mapping=None, part_opt=0, merg_opt=0):
    _csr_lengths(m, n, nnz, csrVal, csrRowPtr, csrColIndex, x, y)
    nm = None if numa_mapping is None else np.ascontiguousarray(numa_mapping, dtype=np.int32)
    return _done(load().spMV_mgpu_v1_numa(m, n, nnz, _scalar(alpha), _d(csrVal), _i(csrRowPtr),
                                          _i(csrColIndex), _d(x), _scalar(beta), _d(y), ngpu,
                                          kernel, _i(nm), part_opt, merg_opt))


def spMV_mgpu_v1_numa_csc(m, n, nnz, alpha, cscVal, cscColPtr, cscRowIndex, x, beta, y, ngpu=1,
                          kernel=1, numa_mapping=None, part_opt=0, merg_opt=0):
    _csc_lengths(m, n, nnz, cscVal, cscColPtr, cscRowIndex, x, y)
    nm = None if numa_mapping is None else np.ascontiguousarray(numa_mapping, dtype=np.int32)
    return _done(load().spMV_mgpu_v1_numa_csc(m, n, nnz, _scalar(alpha), _d(cscVal),
                                              _i(cscColPtr), _i(cscRowIndex), _d(x),
                                              _scalar(beta), _d(y), ngpu, kernel, _i(nm),
                                              part_opt, merg_opt))


def spMV_mgpu_v1_numa_coo(m, n, nnz, alpha, cooVal, cooRowIdx, cooColIdx, x, beta, y, ngpu=1,
                          kernel=1, numa_mapping=None, part_opt=0, merg_opt=0):
    _coo_lengths(m, n, nnz, cooVal, cooRowIdx, cooColIdx, x, y)
    nm = None if numa_mapping is None else np.ascontiguousarray(numa_mapping, dtype=np.int32)
    return _done(load().spMV_mgpu_v1_numa_coo(m, n, nnz, _scalar(alpha), _d(cooVal),
                                              _i(cooRowIdx), _i(cooColIdx), _d(x),
                                              _scalar(beta), _d(y), ngpu, kernel, _i(nm),
                                              part_opt, merg_opt))


def spMV_mgpu_v2(m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta, y, ngpu=1, kernel=2,
                 nb=1 << 24, copy_of_workspace=1):
    _csr_lengths(m, n, nnz, csrVal, csrRowPtr, csrColIndex, x, y)
    return _done(load().spMV_mgpu_v2(m, n, nnz, _scalar(alpha), _d(csrVal), _i(csrRowPtr),
                                     _i(csrColIndex), _d(x), _scalar(beta), _d(y), ngpu, kernel,
                                     nb, copy_of_workspace))


def spMspV_mgpu_v1(m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta, y, ngpu=1,
                   kernel=2):
    _csr_lengths(m, n, nnz, csrVal, csrRowPtr, csrColIndex, x, y)
    return _done(load().spMspV_mgpu_v1(m, n, nnz, _scalar(alpha), _d(csrVal), _i(csrRowPtr),
                                       _i(csrColIndex), _d(x), _scalar(beta), _d(y), ngpu,
                                       kernel))


def spMspV_mgpu_v2(m, n, nnz, alpha, csrVal, csrRowPtr, csrColIndex, x, beta, y, ngpu=1,
                   kernel=2, nb=1 << 24, copy_of_workspace=1):
    _csr_lengths(m, n, nnz, csrVal, csrRowPtr, csrColIndex, x, y)
    return _done(load().spMspV_mgpu_v2(m, n, nnz, _scalar(alpha), _d(csrVal), _i(csrRowPtr),
                                       _i(csrColIndex), _d(x), _scalar(beta), _d(y), ngpu,
                                       kernel, nb, copy_of_workspace))


def _check_helper() -> None:
    lib = load()
    if lib.sblas_last_status() != 0:
        raise SblasError(lib.sblas_last_status(), lib.sblas_last_error().decode())


def coo2csr(m, n, nnz, cooVal, cooRowIdx, cooColIdx):
    """src/spmv_helper.cu:493-572 -> (csrVal, csrRowPtr, csrColIdx)."""
    _coo_lengths(m, n, nnz, cooVal, cooRowIdx, cooColIdx)
    v = np.empty(nnz, np.float64)
    p = np.empty(m + 1, np.int32)
    c = np.empty(nnz, np.int32)
    load().coo2csr(m, n, nnz, _d(cooVal), _i(cooRowIdx), _i(cooColIdx), _d(v), _i(p), _i(c))
    _check_helper()
    return v, p, c


def coo2csc(m, n, nnz, cooVal, cooRowIdx, cooColIdx):
    """src/spmv_helper.cu:575-642 -> (cscVal, cscColPtr, cscRowIdx)."""
    _coo_lengths(m, n, nnz, cooVal, cooRowIdx, cooColIdx)
    v = np.empty(nnz, np.float64)
    p = np.empty(n + 1, np.int32)
    r = np.empty(nnz, np.int32)
    load().coo2csc(m, n, nnz, _d(cooVal), _i(cooRowIdx), _i(cooColIdx), _d(v), _i(p), _i(r))
    _check_helper()
    return v, p, r


def sortCOORow(m, n, nnz, cooVal, cooRowIdx, cooColIdx) -> None:
    _coo_lengths(m, n, nnz, cooVal, cooRowIdx, cooColIdx)
    load().sortCOORow(m, n, nnz, _d(cooVal), _i(cooRowIdx), _i(cooColIdx))
    _check_helper()


def sortCOOCol(m, n, nnz, cooVal, cooRowIdx, cooColIdx) -> None:
    _coo_lengths(m, n, nnz, cooVal, cooRowIdx, cooColIdx)
    load().sortCOOCol(m, n, nnz, _d(cooVal), _i(cooRowIdx), _i(cooColIdx))
    _check_helper()


def get_row_from_index(n, a, idx) -> int:
    return int(load().get_row_from_index(n, _i(a), idx))


def findFirstInSorted(a, n, key) -> int:
    return int(load().findFirstInSorted(_i(a), n, key))


def findLastInSorted(a, n, key) -> int:
    return int(load().findLastInSorted(_i(a), n, key))


def get_time() -> float:
    return float(load().get_time())
