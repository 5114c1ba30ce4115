"""Full-size configurations on the GPU, checked against the oracle (C, all
host threads) and through size-independent properties.

  power-law 4.0M x 4.0M, ~70M nnz, values 1.0, x ~ U(0,1)   CSR, CSC, COO
  banded FEM 2.0M x 2.0M, ~280M nnz, values N(0,1)           CSR FP64 / FP32 values
"""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 8


def rel_l2(y, ref):
    return float(np.linalg.norm(y - ref) / np.linalg.norm(ref))


@pytest.fixture(scope="module")
def powerlaw(cuda):
    from hpda_sblas_pnnl_gb300 import synth
    a, x = synth.powerlaw(device=cuda)
    assert 68e6 < a.nnz < 72e6          # ~70M after duplicate endpoints are merged
    return a, x


def oracle_y(a, x, alpha=1.0, beta=0.0, y0=None):
    rp, c, v = a.numpy()
    xx = x.cpu().numpy()
    y0 = np.zeros(a.m) if y0 is None else y0
    return O.csr_spmv(a.m, a.n, rp, c, v, xx, y0, alpha, beta, threads=THREADS)


def test_powerlaw_csr_all_kernels(sblas_lib, cuda, powerlaw):
    from hpda_sblas_pnnl_gb300 import ops
    a, x = powerlaw
    ref = oracle_y(a, x)
    for k in (1, 2, 3):
        y = torch.full((a.m,), float("nan"), dtype=torch.float64, device=cuda)
        ops.csrmv(a.rowptr, a.col, a.val, x, y, kernel=k)
        torch.cuda.synchronize()
        yy = y.cpu().numpy()
        assert rel_l2(yy, ref) <= 1e-12
        # values are 1.0: each row sum is a sum of x over the row's columns;
        # checksum of checksums: sum(y) = sum_j colcount_j * x_j
    cc = torch.bincount(a.col.to(torch.int64), minlength=a.n).to(torch.float64)
    assert abs(float(y.sum()) - float((cc * x).sum())) <= 1e-9 * float((cc * x).sum())


def test_powerlaw_alpha_beta_linearity(sblas_lib, cuda, powerlaw):
    """A(2x1 - 3x2) = 2Ax1 - 3Ax2 and y = a*A*x + b*y0 (size-independent)."""
    from hpda_sblas_pnnl_gb300 import ops
    a, x = powerlaw
    g = torch.Generator(device=cuda).manual_seed(9)
    x2 = torch.rand(a.n, generator=g, dtype=torch.float64, device=cuda)
    y0 = torch.rand(a.m, generator=g, dtype=torch.float64, device=cuda)
    y1 = torch.zeros(a.m, dtype=torch.float64, device=cuda)
    y2 = torch.zeros_like(y1)
    y3 = torch.zeros_like(y1)
    ops.csrmv(a.rowptr, a.col, a.val, x, y1)
    ops.csrmv(a.rowptr, a.col, a.val, x2, y2)
    ops.csrmv(a.rowptr, a.col, a.val, 2 * x - 3 * x2, y3)
    lin = 2 * y1 - 3 * y2
    assert float((y3 - lin).norm() / lin.norm()) <= 1e-12
    y4 = y0.clone()
    ops.csrmv(a.rowptr, a.col, a.val, x, y4, alpha=-0.5, beta=1.25)
    exp = -0.5 * y1 + 1.25 * y0
    assert float((y4 - exp).norm() / exp.norm()) <= 1e-12


def test_powerlaw_csc_and_coo(sblas_lib, cuda, powerlaw):
    from hpda_sblas_pnnl_gb300 import ops, synth
    a, x = powerlaw
    ref = oracle_y(a, x)
    colptr, rowidx, cval = synth.csr_to_csc(a)
    y = torch.zeros(a.m, dtype=torch.float64, device=cuda)
    ops.cscmv(colptr, rowidx, cval, x, y)
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), ref) <= 1e-12
    # the device transpose returns the CSR arrays exactly
    rp2, c2, v2 = ops.csc_to_csr(a.m, a.n, colptr, rowidx, cval)
    assert torch.equal(rp2, a.rowptr) and torch.equal(c2, a.col) and torch.equal(v2, a.val)
    row = synth.csr_to_coo_rows(a)
    y = torch.zeros(a.m, dtype=torch.float64, device=cuda)
    ops.coomv(row, a.col, a.val, x, y)
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), ref) <= 1e-12


def test_banded_fp64_and_fp32_values(sblas_lib, cuda):
    from hpda_sblas_pnnl_gb300 import ops, synth
    a, x = synth.banded_fem(device=cuda)
    assert 260e6 < a.nnz < 300e6
    ref = oracle_y(a, x)
    y = torch.zeros(a.m, dtype=torch.float64, device=cuda)
    ops.csrmv(a.rowptr, a.col, a.val, x, y)
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), ref) <= 1e-12
    # FP32-stored values, FP64 sums: error against the FP64 oracle <= 1e-6
    v32 = a.val.to(torch.float32)
    y32 = torch.zeros_like(y)
    ops.csrmv(a.rowptr, a.col, v32, x, y32)
    torch.cuda.synchronize()
    assert rel_l2(y32.cpu().numpy(), ref) <= 1e-6


@pytest.mark.parametrize("kernel", [2, 3])
def test_host_entry_point_overlapped_chunks(sblas_lib, cuda, kernel):
    """Host-array calls large enough to be copied in row chunks overlapping
    the kernels (6.4M nonzeros): same result as the oracle, with alpha,
    beta and a y that is read, from pinned and from pageable host arrays."""
    from hpda_sblas_pnnl_gb300 import api, synth
    a, x = synth.powerlaw(m=400_000, mean_deg=17.5, seed=12, device=cuda, values="normal")
    assert a.nnz > (1 << 22)
    rp, c, v = a.numpy()
    xx = x.cpu().numpy()
    rng = np.random.default_rng(4)
    y0 = rng.standard_normal(a.m)
    ref = O.csr_spmv(a.m, a.n, rp, c, v, xx, y0, 1.5, -0.5, threads=THREADS)
    for pinned in (True, False):
        arr = (lambda t: torch.from_numpy(t).pin_memory().numpy()) if pinned else (lambda t: t.copy())
        y = arr(y0.copy())
        ret = api.spMV_mgpu_v1(a.m, a.n, a.nnz, 1.5, arr(v), arr(rp), arr(c), arr(xx), -0.5, y,
                               kernel=kernel)
        assert ret.comp_time >= 0 and ret.comm_time > 0
        assert rel_l2(y, ref) <= 1e-12
        y = arr(np.full(a.m, np.nan))
        api.spMV_mgpu_baseline(a.m, a.n, a.nnz, 1.0, arr(v), arr(rp), arr(c), arr(xx), 0.0, y)
        assert rel_l2(y, O.csr_spmv(a.m, a.n, rp, c, v, xx, np.zeros(a.m), threads=THREADS)) <= 1e-12


def test_nnz_at_the_int32_limit(sblas_lib, cuda):
    """Maximum size: 2,147,000,000 nonzeros (int32 row pointers hold at most
    2^31 - 1), 16M rows of 0 to 268 nonzeros (rowptr[i] = floor((i/m)^2 nnz):
    empty rows first).  Values 1, 2, 3 in turn and x in {1, ..., 4}: every
    product and row sum is an integer below 2^53, so the exact y is known in
    any summation order and every kernel (1, 2, 3, the pattern form and the
    batched plan) must match it bit for bit.  About 32 GB on the device."""
    from hpda_sblas_pnnl_gb300 import ops
    nnz, m, n = 2_147_000_000, 16_000_000, 16_000_000
    g = torch.Generator(device=cuda)
    g.manual_seed(31)
    i = torch.arange(m + 1, dtype=torch.float64, device=cuda)
    rp64 = torch.floor((i / m) ** 2 * nnz).to(torch.int64)
    rp64[-1] = nnz
    del i
    rowptr = rp64.to(torch.int32)
    col = torch.randint(0, n, (nnz,), generator=g, dtype=torch.int32, device=cuda)
    val = torch.empty(nnz, dtype=torch.float64, device=cuda)
    step = 1 << 28
    for s in range(0, nnz, step):
        e = min(nnz, s + step)
        val[s:e] = (torch.arange(s, e, device=cuda) % 3 + 1).to(torch.float64)
    x = torch.randint(1, 5, (n,), generator=g, device=cuda).to(torch.float64)
    # exact results by row blocks: prefix sums of the products
    want = torch.empty(m, dtype=torch.float64, device=cuda)
    want_pat = torch.empty(m, dtype=torch.float64, device=cuda)
    rb = 1 << 20
    for r0 in range(0, m, rb):
        r1 = min(m, r0 + rb)
        j0, j1 = int(rp64[r0]), int(rp64[r1])
        xg = x[col[j0:j1].long()]
        lo, hi = rp64[r0:r1] - j0, rp64[r0 + 1:r1 + 1] - j0
        for out, terms in ((want, val[j0:j1] * xg), (want_pat, xg)):
            pre = torch.zeros(j1 - j0 + 1, dtype=torch.float64, device=cuda)
            torch.cumsum(terms, 0, out=pre[1:])
            out[r0:r1] = pre[hi] - pre[lo]
            del pre
        del xg, lo, hi
    assert float(want.max()) < 2.0 ** 53
    y = torch.empty(m, dtype=torch.float64, device=cuda)
    for kernel in (1, 2, 3):
        y.fill_(float("nan"))
        ops.csrmv(rowptr, col, val, x, y, 1.0, 0.0, n=n, kernel=kernel)
        torch.cuda.synchronize()
        assert torch.equal(y, want), kernel
    y.fill_(float("nan"))
    ops.csrmv(rowptr, col, None, x, y, 1.0, 0.0, n=n)
    torch.cuda.synchronize()
    assert torch.equal(y, want_pat)
    y.fill_(float("nan"))
    plan = ops.SpmmPlan(rowptr, col, val, n=n, k=1)
    plan(x, y)
    torch.cuda.synchronize()
    assert torch.equal(y, want)
    del plan, col, val, rowptr, rp64, want, want_pat, y, x
    torch.cuda.empty_cache()
