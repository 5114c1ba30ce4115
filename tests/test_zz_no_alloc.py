"""sblas_dcsrmv_noalloc: the SpMV for callers that cannot call cudaMalloc
(code inside a device-memory pool or caching allocator, services that
reserve all device memory at start-up).  Its scratch is a fixed device array
inside the library, so this checks, through the C ABI, that after a set-up
call (m = 0) the first call and two more in a row allocate no device memory
and give the same result as the workspace-taking entry point and as the
oracle (the reference's CPU loop restated), and that a matrix too large for
the fixed scratch is refused.  Collected last on purpose (file name), so a
run that stops at the first failure has run every other test first; it
also passes alone.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL_L2 = 1e-12


def _p(t):
    return C.c_void_p(t.data_ptr())


def _rel_l2(y, ref):
    return float((y - ref).norm() / ref.norm())


def test_noalloc_matches_workspace_entry_point_on_two_calls(sblas_lib, cuda):
    from hpda_sblas_pnnl_gb300 import ops, synth
    from oracle import oracle as O
    a, x = synth.powerlaw(m=200_000, mean_deg=17.5, seed=12, device=cuda, values="normal")
    g = torch.Generator(device=cuda).manual_seed(5)
    y0 = torch.rand(a.m, generator=g, dtype=torch.float64, device=cuda)
    alpha, beta = 1.25, -0.5

    ref = y0.clone()
    ops.csrmv(a.rowptr, a.col, a.val, x, ref, alpha, beta)   # existing entry point
    rp, c, v = a.numpy()
    truth = torch.from_numpy(O.csr_spmv(a.m, a.n, rp, c, v, x.cpu().numpy(),
                                        y0.cpu().numpy(), alpha, beta))
    outs = [y0.clone(), y0.clone(), y0.clone()]
    stream = C.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)

    def call(y, m=a.m):
        rc = sblas_lib.sblas_dcsrmv_noalloc(m, a.n, a.nnz, alpha, _p(a.val), _p(a.rowptr),
                                            _p(a.col), _p(x), beta, _p(y), stream)
        assert rc == 0, sblas_lib.sblas_last_error().decode()

    # the set-up call (m = 0: resolves the array, loads the kernels), then the
    # first real call and two more in a row, with no device memory taken
    call(outs[0], m=0)
    torch.cuda.synchronize()
    assert torch.equal(outs[0], y0)                           # set-up computes nothing
    free0, _ = torch.cuda.mem_get_info(cuda)
    for y in outs:
        call(y)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(cuda)
    assert free1 == free0, "device memory changed across allocation-free calls"
    assert sblas_lib.sblas_stream_status(stream, 0) == 0
    for y in outs:
        assert _rel_l2(y, ref) <= RTOL_L2
        assert _rel_l2(y.cpu(), truth) <= RTOL_L2


def test_noalloc_refuses_matrices_beyond_its_scratch(sblas_lib, cuda):
    d = torch.zeros(4, dtype=torch.float64, device=cuda)
    i = torch.zeros(4, dtype=torch.int32, device=cuda)
    cap = int(sblas_lib.sblas_noalloc_scratch_bytes())
    assert cap > 0
    big = 2_000_000_000   # scratch for this many nonzeros exceeds the fixed array
    rc = sblas_lib.sblas_dcsrmv_noalloc(1, 1, big, 1.0, _p(d), _p(i), _p(i), _p(d), 0.0, _p(d),
                                        C.c_void_p(0))
    assert rc == -1
    assert b"scratch" in sblas_lib.sblas_last_error()
    np.testing.assert_array_equal(d.cpu().numpy(), np.zeros(4))   # nothing launched
