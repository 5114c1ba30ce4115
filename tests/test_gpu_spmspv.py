"""SpMSpV: the x-zero filter of spMspV_mgpu_v1 / _v2
(src/dspmv_mgpu_v1.cu:19-74, src/dspmv_mgpu_v2.cu:35-101) on the device
(sblas_csr_filter_x, ops.spmspv) and on the host threads (the drop-in
entry points), against the oracle's restatement of the reference's serial
loop (oracle_csr_filter_x).  Filtered matrices bit for bit; products
within relative L2 1e-12."""
import numpy as np
import pytest
import torch

from conftest import golden_cases, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL_L2 = 1e-12


def rel_l2(y, ref):
    den = np.linalg.norm(ref)
    num = np.linalg.norm(np.asarray(y) - ref)
    return num / den if den > 0 else num


def sparse_x(n, density, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, n)
    x[rng.random(n) >= density] = 0.0
    x[rng.random(n) < 0.05 * density] = -0.0      # negative zeros are zeros too
    return x


def t(a, dt, cuda):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=cuda, dtype=dt)


def check_filter(rp, col, val, x, m, cuda):
    from hpda_sblas_pnnl_gb300 import ops
    orp, oc, ov = O.csr_filter_x(m, rp, col, val, x)
    drp, dc, dv = ops.csr_filter_x(t(rp, torch.int32, cuda), t(col, torch.int32, cuda),
                                   t(val, torch.float64, cuda), t(x, torch.float64, cuda))
    np.testing.assert_array_equal(drp.cpu().numpy(), orp)
    np.testing.assert_array_equal(dc.cpu().numpy(), oc)
    assert dv.cpu().numpy().tobytes() == ov.tobytes()
    return orp, oc, ov


@pytest.mark.parametrize("name", golden_cases())
def test_device_filter_matches_reference_loop_on_golden_cases(sblas_lib, cuda, name):
    g = load_golden(name)
    m, n = int(g["m"]), int(g["n"])
    x = g["x"].copy()
    x[::3] = 0.0
    check_filter(g["rowptr"].astype(np.int32), g["col"].astype(np.int32),
                 g["val"].astype(np.float64), x, m, cuda)


@pytest.mark.parametrize("density", [0.0, 0.01, 0.3, 1.0])
def test_filter_and_product_at_scale(sblas_lib, cuda, density):
    """300k-row power-law matrix; x with 0 %, 1 %, 30 % and 100 % nonzeros.
    The device form (filter + tile kernel on the GPU) and the host entry
    points (filter on all host threads) against the oracle."""
    from hpda_sblas_pnnl_gb300 import api, ops, synth
    a, _ = synth.powerlaw(m=300_000, mean_deg=17.5, seed=41, values="normal")
    rp, col, val = a.numpy()
    m, n = a.m, a.n
    x = sparse_x(n, density, 5)
    orp, oc, ov = check_filter(rp, col, val, x, m, cuda)
    y0 = np.random.default_rng(6).uniform(-1, 1, m)
    ref = O.csr_spmv(m, n, orp, oc, ov, x, y0.copy(), 1.5, -0.5)
    y = t(y0, torch.float64, cuda)
    ops.spmspv(t(rp, torch.int32, cuda), t(col, torch.int32, cuda), t(val, torch.float64, cuda),
               t(x, torch.float64, cuda), y, 1.5, -0.5)
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), ref) <= RTOL_L2
    for entry in ("v1", "v2"):
        yh = y0.copy()
        if entry == "v1":
            api.spMspV_mgpu_v1(m, n, int(col.size), 1.5, val, rp, col, x, -0.5, yh, kernel=2)
        else:
            api.spMspV_mgpu_v2(m, n, int(col.size), 1.5, val, rp, col, x, -0.5, yh, kernel=2)
        assert rel_l2(yh, ref) <= RTOL_L2, entry


def test_filtered_nonzeros_never_reach_the_product(sblas_lib, cuda):
    """Infinite values at columns where x is zero: the reference's filter
    drops them (finite result); a plain SpMV would give NaN (inf * 0)."""
    from hpda_sblas_pnnl_gb300 import api, ops, synth
    a, _ = synth.powerlaw(m=50_000, mean_deg=12.0, seed=43, values="normal")
    rp, col, val = a.numpy()
    x = sparse_x(a.n, 0.2, 7)
    val = val.copy()
    hit = np.nonzero(x[col] == 0.0)[0][::5]
    val[hit] = np.inf
    orp, oc, ov = check_filter(rp, col, val, x, a.m, cuda)
    ref = O.csr_spmv(a.m, a.n, orp, oc, ov, x, np.zeros(a.m))
    assert np.isfinite(ref).all()
    y = torch.zeros(a.m, dtype=torch.float64, device=cuda)
    ops.spmspv(t(rp, torch.int32, cuda), t(col, torch.int32, cuda), t(val, torch.float64, cuda),
               t(x, torch.float64, cuda), y)
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), ref) <= RTOL_L2
    yh = np.zeros(a.m)
    api.spMspV_mgpu_v1(a.m, a.n, int(col.size), 1.0, val, rp, col, x, 0.0, yh, kernel=3)
    assert np.isfinite(yh).all() and rel_l2(yh, ref) <= RTOL_L2


def test_pattern_filter(sblas_lib, cuda):
    from hpda_sblas_pnnl_gb300 import ops, synth
    a, _ = synth.powerlaw(m=20_000, mean_deg=9.0, seed=44)
    rp, col, val = a.numpy()
    x = sparse_x(a.n, 0.1, 8)
    orp, oc, _ = O.csr_filter_x(a.m, rp, col, val, x)
    drp, dc, dv = ops.csr_filter_x(a.rowptr.to(cuda), a.col.to(cuda), None,
                                   t(x, torch.float64, cuda))
    assert dv is None
    np.testing.assert_array_equal(drp.cpu().numpy(), orp)
    np.testing.assert_array_equal(dc.cpu().numpy(), oc)
