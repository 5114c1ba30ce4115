"""The host-array Python mirror without a GPU: argument plumbing and the
array-length checks in front of the C entry points (a stand-in library
records the calls)."""
import numpy as np
import pytest

from conftest import load_golden
from hpda_sblas_pnnl_gb300 import _lib, api
from test_gpu_parity import ENTRIES, ENTRY_CASES, call_entry, empty_case


class _Recorder:
    """Stands in for libsblas_gb300: every entry point returns a successful
    spmv_ret (helpers return nothing) and is recorded."""

    def __init__(self):
        self.calls = []

    def sblas_last_status(self):
        return 0

    def sblas_set_compat_mode(self, mode):
        pass

    def __getattr__(self, name):
        def fn(*args):
            self.calls.append(name)
            return _lib.SpmvRet()
        return fn


@pytest.fixture
def recorder(monkeypatch):
    r = _Recorder()
    monkeypatch.setattr(api, "load", lambda: r)
    return r


@pytest.mark.parametrize("name", ENTRY_CASES)
def test_parity_cases_pass_the_length_checks(recorder, name):
    g = load_golden(name)
    for entry in ENTRIES:
        call_entry(entry, g, g["y0"].copy())
    for m, n in ((0, 5), (4, 0), (0, 0), (3, 7)):   # the GPU tests' empty shapes
        g = empty_case(m, n)
        for entry in ENTRIES:
            call_entry(entry, g, g["y0"].copy())
    assert len(recorder.calls) == 5 * len(ENTRIES)


def _short(a):
    return a[:-1].copy()


@pytest.mark.parametrize("entry", ENTRIES)
def test_short_arrays_fail_before_the_library(recorder, entry):
    g = load_golden("zipf200")
    # (call_entry takes nnz from col's length: a short col is tested below)
    keys = ["x"] + (["csc_val", "csc_colptr", "csc_row"] if "csc" in entry else
                    ["val", "coo_row"] if "coo" in entry else ["val", "rowptr"])
    for k in keys:
        h = dict(g)
        h[k] = _short(g[k])
        with pytest.raises(_lib.SblasError) as e:
            call_entry(entry, h, g["y0"].copy())
        assert e.value.status == api.SBLAS_ERR_ARG and "needed" in str(e.value)
    with pytest.raises(_lib.SblasError):
        call_entry(entry, g, _short(g["y0"]))
    assert recorder.calls == []


def test_short_index_array_with_explicit_nnz(recorder):
    g = load_golden("zipf200")
    m, n, nnz = int(g["m"]), int(g["n"]), int(g["col"].size)
    with pytest.raises(_lib.SblasError, match="csrColIndex"):
        api.spMV_mgpu_v1(m, n, nnz, 1.0, g["val"], g["rowptr"], _short(g["col"]), g["x"], 0.0,
                         g["y0"].copy())
    with pytest.raises(_lib.SblasError, match="cooColIdx"):
        api.spMV_mgpu_baseline_coo(m, n, nnz, 1.0, g["val"], g["coo_row"], _short(g["col"]),
                                   g["x"], 0.0, g["y0"].copy())
    assert recorder.calls == []


def test_conversion_helpers_check_lengths(recorder):
    g = load_golden("zipf200")
    m, n, nnz = int(g["m"]), int(g["n"]), int(g["col"].size)
    args = [g["val"], g["coo_row"], g["col"]]
    for fn in (api.coo2csr, api.coo2csc, api.sortCOORow, api.sortCOOCol):
        fn(m, n, nnz, *args)
        for i in range(3):
            bad = list(args)
            bad[i] = _short(bad[i])
            with pytest.raises(_lib.SblasError):
                fn(m, n, nnz, *bad)
    assert recorder.calls == ["coo2csr", "coo2csc", "sortCOORow", "sortCOOCol"]


def test_negative_sizes_reach_the_library(recorder):
    """Sizes below zero are the library's to reject (with a status)."""
    g = load_golden("zipf200")
    api.spMV_mgpu_baseline(-1, -1, -1, 1.0, g["val"], g["rowptr"], g["col"], g["x"], 0.0,
                           g["y0"].copy())
    assert recorder.calls == ["spMV_mgpu_baseline"]
