"""GPU parity against cuSPARSE, the library behind the reference's kernels 1
and 2 (cusparseDcsrmv / cusparseDcsrmv_mp at src/dspmv_mgpu_v1.cu:256-278,
removed in CUDA 13).  Its CSR SpMV / SpMM successor is reached here through
torch's sparse-CSR matmul, as a checker only: the library under test never
calls cuSPARSE.

Two things are pinned: cuSPARSE agrees with the reference's own CPU loop
(the golden fixtures) within the FP64 bar, and this library's kernels agree
with cuSPARSE within the same bar.  Tolerance: relative L2 <= 1e-12; the
reference's 'g' matrix (small integers) bit for bit."""
import numpy as np
import pytest
import torch

from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu

RTOL_L2 = 1e-12


def rel_l2(y, ref):
    den = np.linalg.norm(ref)
    num = np.linalg.norm(np.asarray(y) - ref)
    return num / den if den > 0 else num


def cusparse_mv(rowptr, col, val, m, n, x, y0, alpha, beta):
    """alpha * (A @ x) + beta * y0 with A @ x from cuSPARSE (FP64).  The CSR
    invariants are checked before cuSPARSE sees the arrays."""
    a = torch.sparse_csr_tensor(rowptr, col, val, size=(m, n), check_invariants=True)
    ax = a @ x
    return alpha * ax + beta * y0 if beta != 0.0 else alpha * ax


def nonempty_cases():
    out = []
    for name in golden_cases():
        g = load_golden(name)
        if int(g["m"]) > 0 and int(g["n"]) > 0 and g["col"].size > 0:
            out.append(name)
    return out


def dev(g, cuda):
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(device=cuda, dtype=dt)
    return (t(g["rowptr"], torch.int32), t(g["col"], torch.int32), t(g["val"], torch.float64),
            t(g["x"], torch.float64), t(g["y0"], torch.float64))


@pytest.mark.parametrize("name", nonempty_cases())
def test_cusparse_agrees_with_reference_cpu_loop(cuda, name):
    g = load_golden(name)
    rp, c, v, x, y0 = dev(g, cuda)
    y = cusparse_mv(rp, c, v, int(g["m"]), int(g["n"]), x, y0, float(g["alpha"]),
                    float(g["beta"]))
    torch.cuda.synchronize()
    if name == "g200":
        np.testing.assert_array_equal(y.cpu().numpy(), g["y_ref_csr"])
    else:
        assert rel_l2(y.cpu().numpy(), g["y_ref_csr"]) <= RTOL_L2


@pytest.mark.parametrize("name", nonempty_cases())
@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_kernels_match_cusparse_on_golden_cases(sblas_lib, cuda, name, kernel):
    from hpda_sblas_pnnl_gb300 import ops
    g = load_golden(name)
    rp, c, v, x, y0 = dev(g, cuda)
    alpha, beta = float(g["alpha"]), float(g["beta"])
    ref = cusparse_mv(rp, c, v, int(g["m"]), int(g["n"]), x, y0, alpha, beta)
    y = y0.clone()
    ops.csrmv(rp, c, v, x, y, alpha, beta, n=int(g["n"]), kernel=kernel)
    torch.cuda.synchronize()
    if name == "g200":
        np.testing.assert_array_equal(y.cpu().numpy(), ref.cpu().numpy())
    else:
        assert rel_l2(y.cpu().numpy(), ref.cpu().numpy()) <= RTOL_L2


def synthetic(kind, cuda):
    from hpda_sblas_pnnl_gb300 import synth
    if kind == "powerlaw":
        a, x = synth.powerlaw(m=300_000, mean_deg=17.5, seed=31, device=cuda, values="normal")
    else:
        a, x = synth.banded_fem(m=60_000, per_row=140, band=6_000, seed=32, device=cuda)
    return a, x


@pytest.mark.parametrize("kind", ["powerlaw", "banded"])
def test_tile_kernel_matches_cusparse_at_scale(sblas_lib, cuda, kind):
    """Every compiled tile shape, alpha = 1.5, beta = -0.5."""
    from hpda_sblas_pnnl_gb300 import ops
    a, x = synthetic(kind, cuda)
    y0 = torch.randn(a.m, dtype=torch.float64, device=cuda)
    ref = cusparse_mv(a.rowptr, a.col, a.val, a.m, a.n, x, y0, 1.5, -0.5).cpu().numpy()
    for s in ops.compiled_sigmas():
        y = y0.clone()
        ops.csrmv(a.rowptr, a.col, a.val, x, y, 1.5, -0.5, n=a.n, sigma=s)
        torch.cuda.synchronize()
        assert rel_l2(y.cpu().numpy(), ref) <= RTOL_L2, s


@pytest.mark.parametrize("k", [4, 16])
def test_spmm_matches_cusparse(sblas_lib, cuda, k):
    """Several right-hand sides: the batched kernel's single-matrix plan
    against cuSPARSE SpMM."""
    from hpda_sblas_pnnl_gb300 import ops
    a, _ = synthetic("powerlaw", cuda)
    x = torch.randn((a.n, k), dtype=torch.float64, device=cuda)
    y = torch.empty((a.m, k), dtype=torch.float64, device=cuda)
    plan = ops.SpmmPlan(a.rowptr, a.col, a.val, n=a.n, k=k)
    plan(x, y)
    ref = torch.sparse_csr_tensor(a.rowptr, a.col, a.val, size=(a.m, a.n),
                                  check_invariants=True) @ x
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), ref.cpu().numpy()) <= RTOL_L2
