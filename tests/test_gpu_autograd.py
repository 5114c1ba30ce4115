"""GPU checks of the differentiable form (hpda_sblas_pnnl_gb300.autograd):
forward and both adjoints against the oracle (oracle_csr_spmm, _spmm_t,
_sddmm), FP64 central finite differences (eps = 1e-6) on sampled entries,
and a dense torch gradient on a 2000-row matrix."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL_L2 = 1e-12


def rel_l2(y, ref):
    den = np.linalg.norm(ref)
    num = np.linalg.norm(np.asarray(y) - ref)
    return num / den if den > 0 else num


def matrix(cuda, m=20_000, deg=20.0, seed=21):
    from hpda_sblas_pnnl_gb300 import synth
    a, _ = synth.powerlaw(m=m, mean_deg=deg, dmax=min(20_000, m), seed=seed, device=cuda,
                          values="normal")
    return a


def test_transpose_structure_matches_scipy(sblas_lib, cuda):
    sp = pytest.importorskip("scipy.sparse")
    from hpda_sblas_pnnl_gb300 import ops
    a = matrix(cuda, m=5_000, deg=9.0)
    rp, c, v = a.numpy()
    t_rp, t_c, perm = ops.csr_transpose(a.m, a.n, a.rowptr, a.col)
    torch.cuda.synchronize()
    at = sp.csr_matrix((v, c, rp), shape=(a.m, a.n)).T.tocsr()
    at.sort_indices()
    np.testing.assert_array_equal(t_rp.cpu().numpy(), at.indptr)
    np.testing.assert_array_equal(t_c.cpu().numpy(), at.indices)
    np.testing.assert_array_equal(v[perm.cpu().numpy()], at.data)
    # the values of A^T gathered on the device, FP64 and FP32
    for dt in (torch.float64, torch.float32):
        src = a.val.to(dt)
        out = torch.empty_like(src)
        ops.gather_values(src, perm, out)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), src.cpu().numpy()[perm.cpu().numpy()])


@pytest.mark.parametrize("k", [1, 4, 16])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_forward_and_adjoints_match_oracle(sblas_lib, cuda, k, dtype):
    from hpda_sblas_pnnl_gb300 import autograd
    a = matrix(cuda)
    rp, c = a.rowptr.cpu().numpy(), a.col.cpu().numpy()
    val = a.val.to(dtype).requires_grad_(True)
    shape_x = (a.n, k) if k > 1 else (a.n,)
    x = torch.randn(shape_x, dtype=torch.float64, device=cuda, requires_grad=True)
    op = autograd.CsrOperator(a.rowptr, a.col, a.n, k, value_dtype=dtype)
    y = autograd.spmm(op, val, x)
    w = torch.randn_like(y)
    (y * w).sum().backward()
    torch.cuda.synchronize()
    v64 = val.detach().double().cpu().numpy()
    xn, wn = x.detach().cpu().numpy(), w.cpu().numpy()
    yref = O.csr_spmm(a.m, a.n, rp, c, v64, xn, np.zeros(y.shape), 1.0, 0.0)
    assert rel_l2(y.detach().cpu().numpy(), yref) <= RTOL_L2
    dxref = O.csr_spmm_t(a.m, a.n, rp, c, v64, wn)
    assert rel_l2(x.grad.cpu().numpy(), dxref) <= RTOL_L2
    dvref = O.csr_sddmm(a.m, a.n, rp, c, wn, xn)
    if dtype == torch.float64:
        assert rel_l2(val.grad.cpu().numpy(), dvref) <= RTOL_L2
    else:   # FP64 products and sums, rounded once to FP32
        assert rel_l2(val.grad.cpu().numpy().astype(np.float64), dvref) <= 1e-7


def test_central_finite_differences(sblas_lib, cuda):
    """FP64, eps = 1e-6, 200 sampled values and 200 sampled entries of X."""
    from hpda_sblas_pnnl_gb300 import autograd
    a = matrix(cuda, m=4_000, deg=12.0, seed=5)
    k = 4
    op = autograd.CsrOperator(a.rowptr, a.col, a.n, k)
    val = a.val.clone().requires_grad_(True)
    x = torch.randn((a.n, k), dtype=torch.float64, device=cuda, requires_grad=True)
    w = torch.randn((a.m, k), dtype=torch.float64, device=cuda)
    loss = lambda v, xx: float((op.forward(v, xx) * w).sum())
    (autograd.spmm(op, val, x) * w).sum().backward()
    eps = 1e-6
    rng = np.random.default_rng(3)
    for p in rng.choice(a.nnz, 200, replace=False):
        vp, vm = val.detach().clone(), val.detach().clone()
        vp[p] += eps
        vm[p] -= eps
        fd = (loss(vp, x.detach()) - loss(vm, x.detach())) / (2 * eps)
        assert abs(fd - float(val.grad[p])) <= 1e-5 * max(1.0, abs(fd)), p
    flat = rng.choice(a.n * k, 200, replace=False)
    for q in flat:
        i, j = divmod(int(q), k)
        xp, xm = x.detach().clone(), x.detach().clone()
        xp[i, j] += eps
        xm[i, j] -= eps
        fd = (loss(val.detach(), xp) - loss(val.detach(), xm)) / (2 * eps)
        assert abs(fd - float(x.grad[i, j])) <= 1e-5 * max(1.0, abs(fd)), (i, j)


def test_dense_reference_gradient(sblas_lib, cuda):
    """2000-row matrix: gradients equal torch's dense FP64 autograd."""
    from hpda_sblas_pnnl_gb300 import autograd, synth
    a = matrix(cuda, m=2_000, deg=20.0, seed=8)
    k = 8
    rows = synth.csr_to_coo_rows(a).long()
    cols = a.col.long()
    val = a.val.clone().requires_grad_(True)
    x = torch.randn((a.n, k), dtype=torch.float64, device=cuda, requires_grad=True)
    w = torch.randn((a.m, k), dtype=torch.float64, device=cuda)
    op = autograd.CsrOperator(a.rowptr, a.col, a.n, k)
    (autograd.spmm(op, val, x) * w).sum().backward()
    val_d = a.val.clone().requires_grad_(True)
    x_d = x.detach().clone().requires_grad_(True)
    dense = torch.zeros((a.m, a.n), dtype=torch.float64, device=cuda).index_put((rows, cols), val_d)
    ((dense @ x_d) * w).sum().backward()
    torch.cuda.synchronize()
    assert rel_l2(val.grad.cpu().numpy(), val_d.grad.cpu().numpy()) <= RTOL_L2
    assert rel_l2(x.grad.cpu().numpy(), x_d.grad.cpu().numpy()) <= RTOL_L2


def test_gradcheck_small(sblas_lib, cuda):
    from hpda_sblas_pnnl_gb300 import autograd
    a = matrix(cuda, m=40, deg=5.0, seed=2)
    op = autograd.CsrOperator(a.rowptr, a.col, a.n, 2)
    val = a.val.clone().requires_grad_(True)
    x = torch.randn((a.n, 2), dtype=torch.float64, device=cuda, requires_grad=True)
    assert torch.autograd.gradcheck(lambda v, xx: autograd.spmm(op, v, xx), (val, x),
                                    eps=1e-6, atol=1e-7)


def test_pattern_operator_differentiates_x_only(sblas_lib, cuda):
    from hpda_sblas_pnnl_gb300 import autograd
    a = matrix(cuda, m=3_000, deg=7.0, seed=4)
    op = autograd.CsrOperator(a.rowptr, a.col, a.n, 1, value_dtype=None)
    x = torch.rand(a.n, dtype=torch.float64, device=cuda, requires_grad=True)
    y = autograd.spmm(op, None, x)
    w = torch.randn_like(y)
    (y * w).sum().backward()
    rp, c = a.rowptr.cpu().numpy(), a.col.cpu().numpy()
    yref = O.csr_spmv(a.m, a.n, rp, c, np.ones(a.nnz), x.detach().cpu().numpy(), np.zeros(a.m))
    assert rel_l2(y.detach().cpu().numpy(), yref) <= RTOL_L2
    dxref = O.csr_spmm_t(a.m, a.n, rp, c, None, w.cpu().numpy())
    assert rel_l2(x.grad.cpu().numpy(), dxref) <= RTOL_L2
