"""The Python side of the device ops without a GPU: argument checks and
plumbing up to the library call.  CPU tensors stand in for device tensors
and a recorder stands in for libsblas_gb300 (every call succeeds and does
nothing), so this covers the checks in front of the kernels, not the
kernels."""
import contextlib

import pytest
import torch

from hpda_sblas_pnnl_gb300 import _lib, ops, synth


class _Recorder:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def fn(*args):
            self.calls.append(name)
            if name == "sblas_tile_sigma_count":
                return 1
            if name in ("sblas_tile_sigma_at", "sblas_default_sigma", "sblas_csr5_sigma"):
                return 11
            return 0
        return fn


def _cpu_device(*ts):
    dev = None
    for t in ts:
        if t is None:
            continue
        if not t.is_contiguous():
            raise ValueError("sblas ops take contiguous tensors")
        dev = t.device if dev is None else dev
    return dev


@pytest.fixture
def lib(monkeypatch):
    r = _Recorder()
    monkeypatch.setattr(_lib, "load", lambda *a, **k: r)
    monkeypatch.setattr(ops, "_require_cuda", _cpu_device)
    monkeypatch.setattr(ops, "_stream_ptr", lambda dev: None)
    monkeypatch.setattr(torch.cuda, "device", lambda dev: contextlib.nullcontext())
    return r


@pytest.fixture(scope="module")
def mat():
    a, x = synth.powerlaw(m=2_000, mean_deg=6.0, dmax=200, seed=3, values="normal")
    return a, x


def test_valid_calls_reach_the_library(lib, mat):
    a, x = mat
    y = torch.zeros(a.m, dtype=torch.float64)
    ops.csrmv(a.rowptr, a.col, a.val, x, y)
    ops.csrmv(a.rowptr, a.col, a.val.float(), x, y, n=a.n)
    ops.csrmv(a.rowptr, a.col, None, x, y)
    row = synth.csr_to_coo_rows(a)
    ops.coomv(row, a.col, a.val, x, y)
    ops.coomv(row, a.col, a.val, x, y, rowptr_work=torch.empty(a.m + 1, dtype=torch.int32))
    colptr, rowidx, cval = synth.csr_to_csc(a)
    ops.csc_to_csr(a.m, a.n, colptr, rowidx, cval)
    ops.cscmv(colptr, rowidx, cval, x, y)
    plan = ops.CsrPlan(a.rowptr, a.col, a.val, n=a.n)
    plan(x, y)
    ops.CsrPlan(a.rowptr, a.col, None)(x, y)
    for k in (1, 8, 16):
        sp = ops.SpmmPlan(a.rowptr, a.col, a.val, n=a.n, k=k)
        xk = torch.zeros((a.n, k) if k > 1 else (a.n,), dtype=torch.float64)
        yk = torch.zeros((a.m, k) if k > 1 else (a.m,), dtype=torch.float64)
        sp(xk, yk)
        sp(xk, yk, val=a.val.clone())
        sp.sddmm(yk, xk, torch.empty(a.nnz, dtype=torch.float64))
        sp.close()
    t_rp, t_c, perm = ops.csr_transpose(a.m, a.n, a.rowptr, a.col)
    ops.gather_values(a.val, perm, torch.empty_like(a.val))
    ops.csr_filter_x(a.rowptr, a.col, a.val, x)
    ops.csr_filter_x(a.rowptr, a.col, None, x)
    for name in ("sblas_dcsrmv", "sblas_dcoomv", "sblas_csc_to_csr", "sblas_csr_analyse",
                 "sblas_dcsrmv_analysed", "sblas_batch_plan_create", "sblas_batch_spmm_xy",
                 "sblas_batch_sddmm", "sblas_csr_transpose", "sblas_gather_values",
                 "sblas_csr_filter_x"):
        assert name in lib.calls, name


def _rejected(lib, exc, fn, *args, **kw):
    before = len(lib.calls)
    with pytest.raises(exc):
        fn(*args, **kw)
    kernels = [c for c in lib.calls[before:] if not c.endswith(("_bytes", "sigma"))]
    assert kernels == [], kernels


def test_bad_arguments_fail_before_the_kernels(lib, mat):
    a, x = mat
    y = torch.zeros(a.m, dtype=torch.float64)
    short_val = a.val[:-1].clone()
    _rejected(lib, ValueError, ops.csrmv, a.rowptr, a.col, short_val, x, y)
    _rejected(lib, ValueError, ops.csrmv, a.rowptr, a.col, a.val, x[:-1].clone(), y, n=a.n)
    row = synth.csr_to_coo_rows(a)
    _rejected(lib, TypeError, ops.coomv, row, a.col, a.val.float(), x, y)
    _rejected(lib, TypeError, ops.coomv, row.long(), a.col, a.val, x, y)
    _rejected(lib, ValueError, ops.coomv, row[:-1].clone(), a.col, a.val, x, y)
    _rejected(lib, ValueError, ops.coomv, row, a.col, short_val, x, y)
    _rejected(lib, ValueError, ops.coomv, row, a.col, a.val, x, y,
              rowptr_work=torch.empty(a.m, dtype=torch.int32))
    colptr, rowidx, cval = synth.csr_to_csc(a)
    _rejected(lib, ValueError, ops.csc_to_csr, a.m, a.n, colptr[:-1].clone(), rowidx, cval)
    _rejected(lib, TypeError, ops.csc_to_csr, a.m, a.n, colptr, rowidx, cval.float())
    _rejected(lib, TypeError, ops.CsrPlan, a.rowptr.long(), a.col, a.val)
    _rejected(lib, ValueError, ops.CsrPlan, a.rowptr, a.col, short_val)
    plan = ops.CsrPlan(a.rowptr, a.col, a.val)
    _rejected(lib, ValueError, plan, x, y[:-1].clone())
    _rejected(lib, TypeError, plan, x.float(), y)
    sp = ops.SpmmPlan(a.rowptr, a.col, a.val, n=a.n, k=16)
    x1 = torch.zeros(a.n, dtype=torch.float64)
    y16 = torch.zeros((a.m, 16), dtype=torch.float64)
    _rejected(lib, ValueError, sp, x1, y16)                  # 1-D x for k = 16
    _rejected(lib, ValueError, sp, torch.zeros((a.n, 8), dtype=torch.float64), y16)
    _rejected(lib, ValueError, sp.sddmm, y16, torch.zeros((a.n, 16), dtype=torch.float64),
              torch.empty(a.nnz - 1, dtype=torch.float64))
    _rejected(lib, ValueError, ops.BatchPlan, [(a.rowptr, a.col, short_val)],
              [torch.zeros((a.n, 4), dtype=torch.float64)],
              [torch.zeros((a.m, 4), dtype=torch.float64)], 4)
    _rejected(lib, ValueError, ops.csr_transpose, a.m + 1, a.n, a.rowptr, a.col)
    t_rp, t_c, perm = ops.csr_transpose(a.m, a.n, a.rowptr, a.col)
    _rejected(lib, TypeError, ops.gather_values, a.val, perm, torch.empty_like(a.val.float()))
    _rejected(lib, ValueError, ops.gather_values, a.val, perm, short_val)
    _rejected(lib, TypeError, ops.csr_filter_x, a.rowptr, a.col, a.val, x.float())
    _rejected(lib, ValueError, ops.csr_filter_x, a.rowptr, a.col, short_val, x)
