"""Failure detection of the tile kernels, exercised without faulting the GPU.

Every wait inside the tile kernels is bounded; a launch that gives up stops
early and reports SBLAS_ERR_TIMEOUT (the reference just prints and exits,
include/detail/cuda/helper_cuda.h:583-595).  The tests shorten the limit to
a few milliseconds and hold the producer warp back through the library's
test hook, so the staged-tile barrier that the compute and epilogue warps
wait on is never completed (a flag that nothing sets).  The error must
reach the caller on the asynchronous path (sblas_stream_status), the
synchronous drop-in path (spMV_mgpu_baseline returns failure) and the
allocation-free path; afterwards, at the default limit, the same calls give
the oracle's result again on the same context.
"""
import ctypes as C
import time

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SBLAS_ERR_TIMEOUT = -9


def _p(t):
    return C.c_void_p(t.data_ptr())


@pytest.fixture()
def stalled(sblas_lib):
    """Short waits and a held-back producer for the test's body only."""
    sblas_lib.sblas_set_wait_limit_ns(2_000_000)     # 2 ms
    sblas_lib.sblas_test_hold_producer(1)
    try:
        yield sblas_lib
    finally:
        sblas_lib.sblas_test_hold_producer(0)
        sblas_lib.sblas_set_wait_limit_ns(0)


def _matrix(cuda):
    from hpda_sblas_pnnl_gb300 import synth
    from oracle import oracle as O
    a, x = synth.powerlaw(m=60_000, mean_deg=12.0, seed=41, device=cuda, values="normal")
    rp, c, v = a.numpy()
    ref = O.csr_spmv(a.m, a.n, rp, c, v, x.cpu().numpy(), np.zeros(a.m))
    return a, x, ref


def _rel(y, ref):
    return float(np.linalg.norm(y - ref) / np.linalg.norm(ref))


def test_device_path_reports_timeout_and_recovers(sblas_lib, cuda):
    from hpda_sblas_pnnl_gb300 import _lib, ops
    a, x, ref = _matrix(cuda)
    stream = C.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    assert sblas_lib.sblas_stream_status(stream, 1) == 0        # clean start
    sblas_lib.sblas_set_wait_limit_ns(2_000_000)
    sblas_lib.sblas_test_hold_producer(1)
    try:
        y = torch.zeros(a.m, dtype=torch.float64, device=cuda)
        t0 = time.perf_counter()
        ops.csrmv(a.rowptr, a.col, a.val, x, y)                 # launches fine
        rc = sblas_lib.sblas_stream_status(stream, 0)
        waited = time.perf_counter() - t0
        assert rc == SBLAS_ERR_TIMEOUT, sblas_lib.sblas_last_error().decode()
        assert b"bounded wait" in sblas_lib.sblas_last_error()
        assert waited < 5.0                                     # returned, did not hang
        # the word is sticky until cleared
        with pytest.raises(_lib.SblasError) as ei:
            ops.check_device(cuda, clear=True)
        assert ei.value.status == SBLAS_ERR_TIMEOUT
        assert sblas_lib.sblas_stream_status(stream, 0) == 0
        # an analysed plan reports the same way
        plan = ops.CsrPlan(a.rowptr, a.col, a.val)
        plan(x, y)
        assert sblas_lib.sblas_stream_status(stream, 1) == SBLAS_ERR_TIMEOUT
    finally:
        sblas_lib.sblas_test_hold_producer(0)
        sblas_lib.sblas_set_wait_limit_ns(0)
    # default limit, same context: correct again, and no error recorded
    y = torch.zeros(a.m, dtype=torch.float64, device=cuda)
    ops.csrmv(a.rowptr, a.col, a.val, x, y)
    ops.check_device(cuda)
    assert _rel(y.cpu().numpy(), ref) <= 1e-12
    plan(x, y)
    ops.check_device(cuda)
    assert _rel(y.cpu().numpy(), ref) <= 1e-12


def test_dropin_path_returns_failure_on_timeout(stalled, cuda):
    from hpda_sblas_pnnl_gb300 import _lib, api
    lib = stalled
    for m in (60_000, 400_000):   # the plain path and the chunked (pipelined) one
        from hpda_sblas_pnnl_gb300 import synth
        from oracle import oracle as O
        a, x = synth.powerlaw(m=m, mean_deg=12.0, seed=43, device=cuda, values="normal")
        rp, c, v = (np.ascontiguousarray(t) for t in a.numpy())
        xh = x.cpu().numpy()
        y = np.zeros(a.m)
        lib.sblas_test_hold_producer(1)
        lib.sblas_set_wait_limit_ns(2_000_000)
        with pytest.raises(_lib.SblasError) as ei:
            api.spMV_mgpu_baseline(a.m, a.n, a.nnz, 1.0, v, rp, c, xh, 0.0, y)
        assert ei.value.status == SBLAS_ERR_TIMEOUT
        assert "bounded wait" in str(ei.value)
        lib.sblas_test_hold_producer(0)
        lib.sblas_set_wait_limit_ns(0)
        lib.sblas_stream_status(C.c_void_p(0), 1)      # clear the sticky word
        r = api.spMV_mgpu_baseline(a.m, a.n, a.nnz, 1.0, v, rp, c, xh, 0.0, y)
        assert not r.failed()
        ref = O.csr_spmv(a.m, a.n, rp, c, v, xh, np.zeros(a.m))
        assert _rel(y, ref) <= 1e-12


def test_noalloc_path_reports_timeout(stalled, cuda):
    a, x, ref = _matrix(cuda)
    lib = stalled
    stream = C.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    lib.sblas_stream_status(stream, 1)
    y = torch.zeros(a.m, dtype=torch.float64, device=cuda)
    rc = lib.sblas_dcsrmv_noalloc(a.m, a.n, a.nnz, 1.0, _p(a.val), _p(a.rowptr), _p(a.col),
                                  _p(x), 0.0, _p(y), stream)
    assert rc == 0
    assert lib.sblas_stream_status(stream, 1) == SBLAS_ERR_TIMEOUT
    lib.sblas_test_hold_producer(0)
    lib.sblas_set_wait_limit_ns(0)
    rc = lib.sblas_dcsrmv_noalloc(a.m, a.n, a.nnz, 1.0, _p(a.val), _p(a.rowptr), _p(a.col),
                                  _p(x), 0.0, _p(y), stream)
    assert rc == 0
    assert lib.sblas_stream_status(stream, 1) == 0
    assert _rel(y.cpu().numpy(), ref) <= 1e-12
