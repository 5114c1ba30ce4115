"""The C-ABI library: it builds for sm_103a, loads without a GPU, exports
every symbol include/*.h declares, and its host-only logic matches the
oracle.  No GPU compute here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT, load_golden
from oracle import oracle as O


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = "\n".join(l for l in h.read_text().splitlines() if not l.startswith("#"))
        for m in re.finditer(r"SBLAS_API\s+[\w\s\*]*?\b(\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_reference_entry_points():
    names = set(declared_symbols())
    for ref in ("spMV_mgpu_baseline", "spMV_mgpu_baseline_csc", "spMV_mgpu_baseline_coo",
                "spMV_mgpu_v1", "spMV_mgpu_v1_numa", "spMV_mgpu_v1_numa_csc",
                "spMV_mgpu_v1_numa_coo", "spMV_mgpu_v2", "csr5_kernel", "spMspV_mgpu_v1",
                "spMspV_mgpu_v2", "get_row_from_index", "findFirstInSorted", "findLastInSorted",
                "coo2csr", "coo2csc", "sortCOORow", "sortCOOCol", "get_time"):
        assert ref in names, ref


def test_library_exports_every_declared_symbol(sblas_lib):
    missing = [s for s in declared_symbols() if not hasattr(sblas_lib, s)]
    assert not missing, missing


def test_python_binding_covers_every_declared_symbol():
    from hpda_sblas_pnnl_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES), \
        set(declared_symbols()) - set(_lib.SIGNATURES)


def test_host_search_helpers_match_reference_golden(sblas_lib):
    from hpda_sblas_pnnl_gb300 import api
    g = load_golden("search")
    a = g["a"]
    for k, f, l in zip(g["keys"], g["first"], g["last"]):
        assert api.findFirstInSorted(a, a.size - 1, int(k)) == f
        assert api.findLastInSorted(a, a.size - 1, int(k)) == l
    rp = g["rowptr"]
    for i, r in zip(g["idx"], g["row_of"]):
        assert api.get_row_from_index(rp.size - 1, rp, int(i)) == r


def test_errors_are_statuses_not_exits(sblas_lib):
    """ngpu != 1, bad kernel numbers and bad sizes fail with a status and a
    message (the reference would exit the process)."""
    from hpda_sblas_pnnl_gb300 import api, _lib
    g = load_golden("zipf200")
    y = g["y0"].copy()
    with pytest.raises(_lib.SblasError) as e:
        api.spMV_mgpu_baseline(int(g["m"]), int(g["n"]), int(g["col"].size), 1.0, g["val"],
                               g["rowptr"], g["col"], g["x"], 0.0, y, ngpu=2)
    assert e.value.status == -2 and "ngpu" in str(e.value)
    with pytest.raises(_lib.SblasError):
        api.spMV_mgpu_v1(int(g["m"]), int(g["n"]), int(g["col"].size), 1.0, g["val"],
                         g["rowptr"], g["col"], g["x"], 0.0, y, ngpu=1, kernel=7)
    with pytest.raises(_lib.SblasError):
        api.spMV_mgpu_v2(int(g["m"]), int(g["n"]), int(g["col"].size), 1.0, g["val"],
                         g["rowptr"], g["col"], g["x"], 0.0, y, nb=0)
    rc = sblas_lib.sblas_dcsrmv(9, 10, 10, 0, 1.0, None, 0, None, None, None, 0.0, None, 0,
                                None, 0, None)
    assert rc == -1 and b"kernel" in sblas_lib.sblas_last_error()
    rc = sblas_lib.sblas_dcsrmv(2, -1, 10, 0, 1.0, None, 0, None, None, None, 0.0, None, 0,
                                None, 0, None)
    assert rc == -1
    np.testing.assert_array_equal(y, g["y0"])  # untouched on failure


def test_batch_plan_argument_errors(sblas_lib):
    """Batched-SpMM plan validation happens on the host, before any CUDA
    call: bad counts, uncompiled k or s, null or misaligned pointers."""
    from hpda_sblas_pnnl_gb300 import _lib
    assert [sblas_lib.sblas_batch_default_s(k) for k in (1, 2, 4, 8, 16)] == [16, 16, 8, 8, 4]
    assert sblas_lib.sblas_batch_default_s(3) == 0
    plan = C.c_void_p()
    one = (_lib.BatchMatrix * 1)()
    one[0] = _lib.BatchMatrix(4, 4, 4, 4096, 8192, 12288, 16384, 2, 20480, 2, 1.0, 0.0)
    assert sblas_lib.sblas_batch_plan_create(0, one, 2, 0, 0, None, C.byref(plan)) == -1
    assert sblas_lib.sblas_batch_plan_create(1, one, 3, 0, 0, None, C.byref(plan)) == -7
    assert sblas_lib.sblas_batch_plan_create(1, one, 2, 0, 5, None, C.byref(plan)) == -7
    assert sblas_lib.sblas_batch_plan_create(1, one, 2, 9, 0, None, C.byref(plan)) == -1
    bad = (_lib.BatchMatrix * 1)()
    bad[0] = _lib.BatchMatrix(4, 4, 4, 4096, None, 12288, 16384, 2, 20480, 2, 1.0, 0.0)
    assert sblas_lib.sblas_batch_plan_create(1, bad, 2, 0, 0, None, C.byref(plan)) == -1
    bad[0] = _lib.BatchMatrix(4, 4, 4, 4096, 8192, 12288, 16392, 2, 20480, 2, 1.0, 0.0)
    assert sblas_lib.sblas_batch_plan_create(1, bad, 2, 0, 0, None, C.byref(plan)) == -5
    assert b"aligned" in sblas_lib.sblas_last_error()
    bad[0] = _lib.BatchMatrix(4, 4, 4, 4096, 8192, 12288, 16384, 1, 20480, 2, 1.0, 0.0)
    assert sblas_lib.sblas_batch_plan_create(1, bad, 2, 0, 0, None, C.byref(plan)) == -5
    assert plan.value is None
    assert sblas_lib.sblas_batch_spmm(None, None) == -1
    assert sblas_lib.sblas_batch_plan_destroy(None) == 0


def test_compat_switch_and_shapes(sblas_lib):
    sblas_lib.sblas_set_compat_mode(1)
    assert sblas_lib.sblas_get_compat_mode() == 1
    sblas_lib.sblas_set_compat_mode(0)
    assert sblas_lib.sblas_get_compat_mode() == 0
    sig = [sblas_lib.sblas_tile_sigma_at(i) for i in range(sblas_lib.sblas_tile_sigma_count())]
    assert sig and all(s % 2 == 1 for s in sig)
    assert sblas_lib.sblas_default_sigma(4_000_000, 70_000_000) in sig
    # CSR5 sigma rule (include/anonymouslib_cuda.h:294-318), nearest compiled shape
    assert sblas_lib.sblas_csr5_sigma(100, 300) == min(sig, key=lambda s: abs(s - 4))
    assert sblas_lib.sblas_csr5_sigma(100, 1100) == min(sig, key=lambda s: abs(s - 11))
    assert sblas_lib.sblas_tile_workspace_bytes(70_000_000, 0) > 0


def test_build_targets_sm103a():
    from hpda_sblas_pnnl_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in build.ARCH
    assert build.lib_path().exists()
