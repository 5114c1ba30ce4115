"""ctypes binding of libsblas_gb300.so (the C ABI in include/*.h).

The library is the product: there is no Python or CPU fallback.  If the
shared object is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import build as _build

_LIB: C.CDLL | None = None


class SpmvRet(C.Structure):
    """include/spmv_kernel.h:16-57 (spmv_ret): per-phase seconds of one call."""

    _fields_ = [
        ("numa_part_time", C.c_double),
        ("part_time", C.c_double),
        ("comp_time", C.c_double),
        ("comm_time", C.c_double),
        ("merg_time", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}

    def failed(self) -> bool:
        return self.comp_time < 0


class BatchMatrix(C.Structure):
    """include/sblas_gb300.h (sblas_batch_matrix): one matrix of a batch."""

    _fields_ = [
        ("m", C.c_int),
        ("n", C.c_int),
        ("nnz", C.c_longlong),
        ("val", C.c_void_p),
        ("rowptr", C.c_void_p),
        ("col", C.c_void_p),
        ("x", C.c_void_p),
        ("ldx", C.c_int),
        ("y", C.c_void_p),
        ("ldy", C.c_int),
        ("alpha", C.c_double),
        ("beta", C.c_double),
        ("row_ids", C.c_void_p),
        ("val_perm", C.c_void_p),
    ]


class NnzPart(C.Structure):
    """include/sblas_gb300.h (sblas_nnz_part): one part of the v1 nnz split."""

    _fields_ = [(f, C.c_int) for f in ("start_idx", "end_idx", "start_row", "end_row",
                                        "start_flag", "end_flag", "m", "nnz")]


class MMHeader(C.Structure):
    """include/mmio.h (sblas_mm_header): banner and size line of a file."""

    _fields_ = [
        ("m", C.c_int),
        ("n", C.c_int),
        ("nnz", C.c_longlong),
        ("typecode", C.c_char * 4),
        ("reserved", C.c_int),
    ]


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

# name -> (restype, argtypes); every symbol declared in include/*.h
SIGNATURES: dict[str, tuple] = {
    # include/sblas_gb300.h
    "sblas_last_error": (C.c_char_p, []),
    "sblas_last_status": (C.c_int, []),
    "sblas_version": (C.c_char_p, []),
    "sblas_stream_status": (C.c_int, [C.c_void_p, C.c_int]),
    "sblas_cscmv_workspace_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_longlong]),
    "sblas_dcscmv": (C.c_int, [C.c_int, C.c_int, C.c_longlong, C.c_double, _vp, _vp, _vp, _vp,
                               C.c_double, _vp, _vp, C.c_size_t, _vp]),
    "sblas_csc_analyse": (C.c_int, [C.c_int, C.c_int, C.c_longlong, _vp, _vp, _vp, C.c_size_t,
                                    _vp]),
    "sblas_dcscmv_analysed": (C.c_int, [C.c_int, C.c_int, C.c_longlong, C.c_double, _vp, _vp,
                                        C.c_double, _vp, _vp, C.c_size_t, _vp]),
    "sblas_csc_bind_values": (C.c_int, [C.c_int, C.c_int, C.c_longlong, _vp, _vp, C.c_size_t,
                                        _vp]),
    "sblas_nnz_partition": (C.c_int, [C.c_int, C.c_longlong, _ip, C.c_int, C.c_void_p]),
    "sblas_part_rowptr": (C.c_int, [_ip, C.c_void_p, _ip]),
    "sblas_merge_parts": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_double, _dp]),
    "sblas_set_wait_limit_ns": (None, [C.c_ulonglong]),
    "sblas_test_hold_producer": (None, [C.c_int]),
    "sblas_set_compat_mode": (None, [C.c_int]),
    "sblas_get_compat_mode": (C.c_int, []),
    "sblas_tile_workspace_bytes": (C.c_size_t, [C.c_longlong, C.c_int]),
    "sblas_tile_sigma_count": (C.c_int, []),
    "sblas_tile_sigma_at": (C.c_int, [C.c_int]),
    "sblas_default_sigma": (C.c_int, [C.c_int, C.c_longlong]),
    "sblas_csr5_sigma": (C.c_int, [C.c_int, C.c_longlong]),
    "sblas_dcsrmv": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_double, _vp, C.c_int,
                               _vp, _vp, _vp, C.c_double, _vp, C.c_int, _vp, C.c_size_t, _vp]),
    "sblas_csr_analyse": (C.c_int, [C.c_int, C.c_int, C.c_longlong, _vp, C.c_int, _vp,
                                    C.c_size_t, _vp]),
    "sblas_dcsrmv_analysed": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_double, _vp,
                                        C.c_int, _vp, _vp, _vp, C.c_double, _vp, C.c_int, _vp,
                                        C.c_size_t, _vp]),
    "sblas_noalloc_scratch_bytes": (C.c_size_t, []),
    "sblas_dcsrmv_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, _vp, _vp, _vp, _vp,
                                       C.c_double, _vp, _vp]),
    "sblas_dcoomv": (C.c_int, [C.c_int, C.c_int, C.c_longlong, C.c_double, _vp, _vp, _vp, _vp,
                               C.c_double, _vp, _vp, C.c_int, _vp, C.c_size_t, _vp]),
    "sblas_csc_to_csr_workspace_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_longlong]),
    "sblas_csc_to_csr": (C.c_int, [C.c_int, C.c_int, C.c_longlong, _vp, _vp, _vp, _vp, _vp, _vp,
                                   _vp, C.c_size_t, _vp]),
    "sblas_coo_rows_to_rowptr": (C.c_int, [C.c_int, C.c_longlong, _vp, _vp, _vp]),
    "sblas_batch_default_s": (C.c_int, [C.c_int]),
    "sblas_batch_plan_create": (C.c_int, [C.c_int, C.POINTER(BatchMatrix), C.c_int, C.c_int,
                                          C.c_int, _vp, C.POINTER(_vp)]),
    "sblas_batch_plan_destroy": (C.c_int, [_vp]),
    "sblas_batch_plan_info": (C.c_int, [_vp, C.POINTER(C.c_longlong), _ip,
                                        C.POINTER(C.c_size_t)]),
    "sblas_batch_spmm": (C.c_int, [_vp, _vp]),
    "sblas_batch_spmm_xy": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp, C.c_int, C.c_double,
                                      C.c_double, _vp]),
    "sblas_batch_sddmm": (C.c_int, [_vp, _vp, C.c_int, _vp, C.c_int, _vp, _vp]),
    "sblas_csr_transpose_workspace_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_longlong]),
    "sblas_csr_transpose": (C.c_int, [C.c_int, C.c_int, C.c_longlong, _vp, _vp, _vp, _vp, _vp,
                                      _vp, C.c_size_t, _vp]),
    "sblas_gather_values": (C.c_int, [C.c_longlong, C.c_int, _vp, _vp, _vp, _vp]),
    "sblas_zero": (C.c_int, [_vp, C.c_size_t, _vp]),
    "sblas_csr_filter_x_workspace_bytes": (C.c_size_t, [C.c_longlong]),
    "sblas_csr_filter_x": (C.c_int, [C.c_int, C.c_longlong, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                     _vp, C.c_size_t, _vp]),
    # include/spmv_kernel.h (reference signatures)
    "csr5_kernel": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _vp, _vp, _vp, _vp, _dp, _vp, _vp]),
    "spMV_mgpu_baseline": (SpmvRet, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp,
                                     _dp, C.c_int]),
    "spMV_mgpu_baseline_csc": (SpmvRet, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp,
                                         _dp, C.c_int]),
    "spMV_mgpu_baseline_coo": (SpmvRet, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp,
                                         _dp, C.c_int]),
    "spMV_mgpu_v1": (SpmvRet, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp, _dp,
                               C.c_int, C.c_int]),
    "spMV_mgpu_v1_numa": (SpmvRet, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp, _dp,
                                    C.c_int, C.c_int, _ip, C.c_int, C.c_int]),
    "spMV_mgpu_v1_numa_csc": (SpmvRet, [C.c_int, C.c_int, C.c_longlong, _dp, _dp, _ip, _ip, _dp,
                                        _dp, _dp, C.c_int, C.c_int, _ip, C.c_int, C.c_int]),
    "spMV_mgpu_v1_numa_coo": (SpmvRet, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp,
                                        _dp, C.c_int, C.c_int, _ip, C.c_int, C.c_int]),
    "spMV_mgpu_v2": (SpmvRet, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp, _dp,
                               C.c_int, C.c_int, C.c_int, C.c_int]),
    "spMspV_mgpu_v1": (SpmvRet, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp, _dp,
                                 C.c_int, C.c_int]),
    "spMspV_mgpu_v2": (SpmvRet, [C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp, _dp,
                                 C.c_int, C.c_int, C.c_int, C.c_int]),
    "get_row_from_index": (C.c_int, [C.c_int, _ip, C.c_int]),
    "get_time": (C.c_double, []),
    "get_gpu_availble_mem": (C.c_double, [C.c_int]),
    "coo2csr": (None, [C.c_int, C.c_int, C.c_int, _dp, _ip, _ip, _dp, _ip, _ip]),
    "coo2csc": (None, [C.c_int, C.c_int, C.c_int, _dp, _ip, _ip, _dp, _ip, _ip]),
    "sortCOORow": (None, [C.c_int, C.c_int, C.c_int, _dp, _ip, _ip]),
    "sortCOOCol": (None, [C.c_int, C.c_int, C.c_int, _dp, _ip, _ip]),
    "coo2csrGPU": (None, [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "findFirstInSorted": (C.c_int, [_ip, C.c_int, C.c_int]),
    "findLastInSorted": (C.c_int, [_ip, C.c_int, C.c_int]),
    "report_mem_usage": (None, [C.c_int]),
    "report_all_mem_usage": (None, []),
    "print_vec_double": (None, [_dp, C.c_int, C.c_char_p]),
    "print_vec_int": (None, [_ip, C.c_int, C.c_char_p]),
    "print_vec_gpu_double": (None, [_dp, C.c_int, C.c_char_p]),
    "print_vec_gpu_int": (None, [_ip, C.c_int, C.c_char_p]),
    # include/mmio.h (FILE * and MM_typecode passed as plain pointers)
    "mm_read_banner": (C.c_int, [_vp, _vp]),
    "mm_read_mtx_crd_size": (C.c_int, [_vp, _ip, _ip, _ip]),
    "mm_read_mtx_array_size": (C.c_int, [_vp, _ip, _ip]),
    "mm_is_valid": (C.c_int, [C.c_char_p]),
    "mm_typecode_to_str": (_vp, [C.c_char_p]),
    "sblas_mm_read_header": (C.c_int, [C.c_char_p, C.POINTER(MMHeader)]),
    "sblas_mm_read_coo": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_longlong, _vp, _vp, _vp,
                                    C.POINTER(C.c_longlong)]),
}


class SblasError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"sblas status {status}: {msg}")
        self.status = status


def lib_path() -> Path:
    env = os.environ.get("SBLAS_GB300_LIB")
    return Path(env) if env else _build.lib_path()


def load(build_if_missing: bool = False) -> C.CDLL:
    """Loads libsblas_gb300.so; raises if it is absent (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = lib_path()
    if not p.exists():
        if build_if_missing:
            p = _build.build()
        else:
            raise RuntimeError(
                f"{p} is missing: build it with `python -m hpda_sblas_pnnl_gb300.build` "
                "(this package has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(rc: int) -> None:
    if rc != 0:
        lib = load()
        raise SblasError(rc, lib.sblas_last_error().decode())


def last_error() -> str:
    return load().sblas_last_error().decode()
