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
    assert 60e6 < a.nnz < 80e6
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
