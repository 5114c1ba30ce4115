"""GPU parity: the CUDA kernels and the drop-in entry points against the
reference's own CPU results (golden fixtures) and the oracle.

Tolerance: relative L2 error <= 1e-12 against the FP64 reference result
(the bar the task sets; it allows for summation-order differences).  Cases
whose values are small integers (the reference's 'g' matrix) must match
bit for bit.
"""
import numpy as np
import pytest
import torch

from conftest import golden_cases, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL_L2 = 1e-12


def rel_l2(y, ref):
    y = np.asarray(y, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.linalg.norm(ref)
    num = np.linalg.norm(y - ref)
    return num / den if den > 0 else num


def assert_close(y, ref, exact=False):
    if exact:
        np.testing.assert_array_equal(y, ref)
    else:
        assert rel_l2(y, ref) <= RTOL_L2, rel_l2(y, ref)


def dev(g, cuda):
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(device=cuda, dtype=dt)
    return (t(g["rowptr"], torch.int32), t(g["col"], torch.int32), t(g["val"], torch.float64),
            t(g["x"], torch.float64), t(g["y0"], torch.float64))


def sigmas():
    from hpda_sblas_pnnl_gb300 import ops
    return ops.compiled_sigmas()


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_device_csrmv_matches_reference(sblas_lib, cuda, name, kernel):
    from hpda_sblas_pnnl_gb300 import ops
    g = load_golden(name)
    rp, c, v, x, y = dev(g, cuda)
    ops.csrmv(rp, c, v, x, y, float(g["alpha"]), float(g["beta"]), n=int(g["n"]), kernel=kernel)
    torch.cuda.synchronize()
    assert_close(y.cpu().numpy(), g["y_ref_csr"], exact=(name == "g200"))


@pytest.mark.parametrize("name", ["zipf200_ab", "long_row", "empty_rows", "sparse_rows",
                                  "diag3000", "g200"])
def test_every_tile_shape(sblas_lib, cuda, name):
    from hpda_sblas_pnnl_gb300 import ops
    g = load_golden(name)
    for s in sigmas():
        rp, c, v, x, y = dev(g, cuda)
        ops.csrmv(rp, c, v, x, y, float(g["alpha"]), float(g["beta"]), n=int(g["n"]), sigma=s)
        torch.cuda.synchronize()
        assert_close(y.cpu().numpy(), g["y_ref_csr"], exact=(name == "g200"))


def test_beta_zero_ignores_nan_in_y(sblas_lib, cuda):
    from hpda_sblas_pnnl_gb300 import ops
    g = load_golden("zipf200")
    rp, c, v, x, y = dev(g, cuda)
    y.fill_(float("nan"))
    for k in (1, 2, 3):
        ops.csrmv(rp, c, v, x, y, 1.0, 0.0, kernel=k)
        torch.cuda.synchronize()
        assert_close(y.cpu().numpy(), g["y_ref_csr"])


def test_results_are_bit_reproducible(sblas_lib, cuda):
    from hpda_sblas_pnnl_gb300 import ops, synth
    a, x = synth.powerlaw(m=200_000, mean_deg=17.5, seed=5, device=cuda, values="normal")
    outs = []
    for _ in range(3):
        y = torch.zeros(a.m, dtype=torch.float64, device=cuda)
        ops.csrmv(a.rowptr, a.col, a.val, x, y)
        outs.append(y.clone())
    torch.cuda.synchronize()
    assert all(torch.equal(outs[0], o) for o in outs[1:])


# ---- the drop-in entry points (host arrays, reference signatures) ----------

ENTRY_CASES = ["g200", "zipf200", "zipf200_ab", "empty_rows", "long_row", "one", "nnz0",
               "diag3000", "sparse_rows"]


def call_entry(entry, g, y, kernel=2, merg_opt=0):
    from hpda_sblas_pnnl_gb300 import api
    m, n, nnz = int(g["m"]), int(g["n"]), int(g["col"].size)
    a, b = float(g["alpha"]), float(g["beta"])
    if entry == "baseline":
        return api.spMV_mgpu_baseline(m, n, nnz, a, g["val"], g["rowptr"], g["col"], g["x"], b, y)
    if entry == "v1":
        return api.spMV_mgpu_v1(m, n, nnz, a, g["val"], g["rowptr"], g["col"], g["x"], b, y,
                                kernel=kernel)
    if entry == "v1_numa":
        return api.spMV_mgpu_v1_numa(m, n, nnz, a, g["val"], g["rowptr"], g["col"], g["x"], b, y,
                                     kernel=kernel, numa_mapping=[0], part_opt=1,
                                     merg_opt=merg_opt)
    if entry == "v2":
        return api.spMV_mgpu_v2(m, n, nnz, a, g["val"], g["rowptr"], g["col"], g["x"], b, y,
                                kernel=kernel, nb=1000, copy_of_workspace=4)
    if entry == "baseline_csc":
        return api.spMV_mgpu_baseline_csc(m, n, nnz, a, g["csc_val"], g["csc_colptr"],
                                          g["csc_row"], g["x"], b, y)
    if entry == "v1_numa_csc":
        return api.spMV_mgpu_v1_numa_csc(m, n, nnz, a, g["csc_val"], g["csc_colptr"],
                                         g["csc_row"], g["x"], b, y, merg_opt=merg_opt)
    if entry == "baseline_coo":
        return api.spMV_mgpu_baseline_coo(m, n, nnz, a, g["val"], g["coo_row"], g["col"], g["x"],
                                          b, y)
    if entry == "v1_numa_coo":
        return api.spMV_mgpu_v1_numa_coo(m, n, nnz, a, g["val"], g["coo_row"], g["col"], g["x"],
                                         b, y, merg_opt=merg_opt)
    if entry == "spmspv_v1":
        return api.spMspV_mgpu_v1(m, n, nnz, a, g["val"], g["rowptr"], g["col"], g["x"], b, y,
                                  kernel=kernel)
    raise ValueError(entry)


ENTRIES = ["baseline", "v1", "v1_numa", "v2", "baseline_csc", "v1_numa_csc", "baseline_coo",
           "v1_numa_coo", "spmspv_v1"]


@pytest.mark.parametrize("entry", ENTRIES)
@pytest.mark.parametrize("name", ENTRY_CASES)
def test_dropin_entry_points(sblas_lib, name, entry):
    from hpda_sblas_pnnl_gb300 import api
    api.set_compat_mode(0)
    g = load_golden(name)
    kernels = [1, 2, 3] if entry in ("v1", "v2") else [2]
    for k in kernels:
        y = g["y0"].copy()
        r = call_entry(entry, g, y, kernel=k)
        assert r.comp_time >= 0 and r.comm_time >= 0
        ref = g["y_ref_coo"] if "coo" in entry else g["y_ref_csr"]
        assert_close(y, ref, exact=(name == "g200"))


def empty_case(m, n):
    """A matrix without nonzeros: m x n, alpha 2, beta -0.5."""
    rng = np.random.default_rng(m * 10 + n)
    return {"m": np.int64(m), "n": np.int64(n), "alpha": 2.0, "beta": -0.5,
            "rowptr": np.zeros(m + 1, np.int32), "col": np.zeros(0, np.int32),
            "val": np.zeros(0), "x": rng.uniform(-1, 1, n), "y0": rng.uniform(-1, 1, m),
            "csc_val": np.zeros(0), "csc_colptr": np.zeros(n + 1, np.int32),
            "csc_row": np.zeros(0, np.int32), "coo_row": np.zeros(0, np.int32)}


@pytest.mark.parametrize("entry", ENTRIES)
@pytest.mark.parametrize("shape", [(0, 5), (4, 0), (0, 0), (3, 7)])
def test_dropin_entry_points_without_nonzeros(sblas_lib, entry, shape):
    """No rows, no columns, or no nonzeros: y = beta * y0, no failure."""
    from hpda_sblas_pnnl_gb300 import api
    api.set_compat_mode(0)
    g = empty_case(*shape)
    for k in ([1, 2, 3] if entry in ("v1", "v2") else [2]):
        y = g["y0"].copy()
        r = call_entry(entry, g, y, kernel=k)
        assert r.comp_time >= 0
        np.testing.assert_array_equal(y, -0.5 * g["y0"])


def compat_expected(entry, g, kernel=2, merg_opt=0):
    """The reference's ngpu = 1 result where it differs from y = aAx + by:
    nnz-split entry points touch only rows [first, last non-empty]; CSC and
    merg_opt = 0 merges add into y0; kernel 3 computes A*x."""
    m, n = int(g["m"]), int(g["n"])
    a, b = float(g["alpha"]), float(g["beta"])
    y0 = g["y0"]
    if kernel == 3 and entry in ("v1", "v2"):
        a, b = 1.0, 0.0
    full = O.csr_spmv(m, n, g["rowptr"], g["col"], g["val"], g["x"], y0, a, b)
    out = full.copy()
    additive = entry in ("baseline_csc", "v1_numa_csc") or (
        entry in ("v1_numa", "v1_numa_coo") and merg_opt == 0)
    if additive:
        out = y0 + full
    if entry in ("v1", "v1_numa", "v2", "v1_numa_coo") and g["col"].size > 0:
        rp = g["rowptr"]
        lo = O.get_row_from_index(m, rp, 0)
        hi = O.get_row_from_index(m, rp, int(rp[-1]) - 1) + 1
        out[:lo] = y0[:lo]
        out[hi:] = y0[hi:]
    return out


@pytest.mark.parametrize("entry", ["v1", "v1_numa", "v2", "baseline_csc", "v1_numa_csc",
                                   "v1_numa_coo"])
@pytest.mark.parametrize("name", ["empty_rows", "zipf200_ab", "sparse_rows"])
def test_reference_compat_mode(sblas_lib, name, entry):
    from hpda_sblas_pnnl_gb300 import api
    g = load_golden(name)
    api.set_compat_mode(1)
    try:
        for k in ([1, 2, 3] if entry in ("v1", "v2") else [2]):
            for mo in ([0, 1] if "numa" in entry else [0]):
                y = g["y0"].copy()
                call_entry(entry, g, y, kernel=k, merg_opt=mo)
                assert_close(y, compat_expected(entry, g, k, mo))
    finally:
        api.set_compat_mode(0)


def test_host_format_helpers_match_oracle(sblas_lib):
    from hpda_sblas_pnnl_gb300 import api
    rng = np.random.default_rng(1)
    m, n, nnz = 1000, 700, 20000
    row = rng.integers(0, m, nnz).astype(np.int32)
    col = rng.integers(0, n, nnz).astype(np.int32)
    val = rng.normal(size=nnz)
    for fn, ofn in ((api.coo2csr, O.coo2csr), (api.coo2csc, O.coo2csc)):
        got = fn(m, n, nnz, val, row, col)
        exp = ofn(m, n, val, row, col)
        for a, b in zip(got, exp):
            np.testing.assert_array_equal(a, b)   # stable sort: identical arrays
    r2, c2, v2 = row.copy(), col.copy(), val.copy()
    api.sortCOORow(m, n, nnz, v2, r2, c2)
    order = np.argsort(row, kind="stable")
    np.testing.assert_array_equal(r2, row[order])
    np.testing.assert_array_equal(c2, col[order])
    np.testing.assert_array_equal(v2, val[order])
    r3, c3, v3 = row.copy(), col.copy(), val.copy()
    api.sortCOOCol(m, n, nnz, v3, r3, c3)
    order = np.argsort(col, kind="stable")
    np.testing.assert_array_equal(c3, col[order])
    np.testing.assert_array_equal(r3, row[order])


def test_csr5_kernel_device_entry(sblas_lib, cuda):
    """include/spmv_kernel.h:205-209: device arrays, caller's stream."""
    import ctypes as C
    g = load_golden("zipf200_ab")
    rp, c, v, x, y = dev(g, cuda)
    st = torch.cuda.current_stream(cuda).cuda_stream
    a, b = C.c_double(float(g["alpha"])), C.c_double(float(g["beta"]))
    rc = sblas_lib.csr5_kernel(int(g["m"]), int(g["n"]), int(g["col"].size), C.byref(a),
                               C.c_void_p(v.data_ptr()), C.c_void_p(rp.data_ptr()),
                               C.c_void_p(c.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(b),
                               C.c_void_p(y.data_ptr()), C.c_void_p(st))
    assert rc == 0
    torch.cuda.synchronize()
    assert_close(y.cpu().numpy(), g["y_ref_csr"])


# ---- mixed-precision forms: FP32-stored values, pattern-only ---------------

@pytest.mark.parametrize("name", ["zipf200_ab", "long_row", "empty_rows", "sparse_rows",
                                  "diag3000", "g200", "one"])
def test_fp32_values_and_pattern_forms(sblas_lib, cuda, name):
    """FP32-stored values (widened to FP64, products and sums in FP64):
    within 1e-12 of the FP64 result on the FP32-rounded values, and within
    1e-6 of the FP64 oracle.  Pattern-only: every stored entry is 1."""
    from hpda_sblas_pnnl_gb300 import ops
    g = load_golden(name)
    m, n = int(g["m"]), int(g["n"])
    a, b = float(g["alpha"]), float(g["beta"])
    v32 = g["val"].astype(np.float32)
    ref32 = O.csr_spmv(m, n, g["rowptr"], g["col"], v32.astype(np.float64), g["x"], g["y0"], a, b)
    refpat = O.csr_spmv(m, n, g["rowptr"], g["col"], np.ones_like(g["val"]), g["x"], g["y0"], a, b)
    for s in sigmas():
        rp, c, _, x, y = dev(g, cuda)
        v = torch.from_numpy(v32).to(cuda)
        ops.csrmv(rp, c, v, x, y, a, b, n=n, sigma=s)
        torch.cuda.synchronize()
        assert_close(y.cpu().numpy(), ref32)
        assert rel_l2(y.cpu().numpy(), g["y_ref_csr"]) <= 1e-6
        rp, c, _, x, y = dev(g, cuda)
        ops.csrmv(rp, c, None, x, y, a, b, n=n, sigma=s)
        torch.cuda.synchronize()
        assert_close(y.cpu().numpy(), refpat)


def test_fp32_widening_is_exact_for_every_float_class(sblas_lib, cuda):
    """One nonzero per row, x = 1, alpha = 1, beta = 0: y[i] must equal the
    FP32 value widened to FP64 bit for bit, for zeros of both signs,
    subnormals, normals at both ends of the range, infinities and NaN."""
    from hpda_sblas_pnnl_gb300 import ops
    specials = np.array([0.0, -0.0, 1e-45, -1e-45, 1.1754942e-38, 1.17549435e-38, -3.4028235e38,
                         3.4028235e38, np.inf, -np.inf, np.nan, 1.0, -2.5, 3e-39, 65504.0],
                        dtype=np.float32)
    rng = np.random.default_rng(11)
    bits = rng.integers(0, 2**32, size=20_000, dtype=np.uint64).astype(np.uint32)
    vals = np.concatenate([specials, bits.view(np.float32)])
    m = vals.size
    rp = torch.arange(m + 1, dtype=torch.int32, device=cuda)
    c = torch.arange(m, dtype=torch.int32, device=cuda)
    x = torch.ones(m, dtype=torch.float64, device=cuda)
    want = 0.0 + vals.astype(np.float64)    # the row sum starts at +0: -0 + 0 = +0
    for s in sigmas():
        y = torch.zeros(m, dtype=torch.float64, device=cuda)
        ops.csrmv(rp, c, torch.from_numpy(vals).to(cuda), x, y, sigma=s)
        torch.cuda.synchronize()
        got = y.cpu().numpy()
        nan = np.isnan(want)
        assert (np.isnan(got) == nan).all()
        np.testing.assert_array_equal(got[~nan].view(np.uint64), want[~nan].view(np.uint64))


def test_fp32_values_with_subnormals_and_huge_entries(sblas_lib, cuda):
    """Power-law matrix whose FP32 values include subnormals and values near
    the FP32 maximum: the FP64 accumulation matches the oracle to 1e-12."""
    from hpda_sblas_pnnl_gb300 import ops, synth
    a, x = synth.powerlaw(m=20_000, mean_deg=17.5, seed=3, device=cuda, values="normal")
    v32 = a.val.to(torch.float32)
    v32[::101] = 3e-41
    v32[7::1013] = 3e38
    ref = O.csr_spmv(a.m, a.n, a.rowptr.cpu().numpy(), a.col.cpu().numpy(),
                     v32.double().cpu().numpy(), x.cpu().numpy(), np.zeros(a.m))
    y = torch.zeros(a.m, dtype=torch.float64, device=cuda)
    ops.csrmv(a.rowptr, a.col, v32, x, y)
    torch.cuda.synchronize()
    yy = y.cpu().numpy()
    scale = np.abs(ref).max()
    assert rel_l2(yy / scale, ref / scale) <= 1e-12
    small = np.abs(ref) < 1e30
    assert rel_l2(yy[small], ref[small]) <= 1e-12

@pytest.mark.parametrize("nnz", [1, 2, 3, 4, 5, 7, 8, 1000, 1001, 1_000_003])
@pytest.mark.parametrize("offset", [0, 1])
def test_coo_row_pointer_builder(sblas_lib, cuda, nnz, offset):
    """Row pointer of row-sorted COO built on the device (the step before
    the COO SpMV; the reference's coo2csrGPU), against numpy: rows empty at
    the start, middle and end; a 16-byte aligned row array (the four-index
    kernel) and one misaligned by 4 bytes (the one-index kernel)."""
    import ctypes as C
    rng = np.random.default_rng(nnz + offset)
    m = max(8, nnz // 3)
    rows = np.sort(rng.integers(2, m - 2, nnz)).astype(np.int32)
    buf = torch.zeros(nnz + 1, dtype=torch.int32, device=cuda)
    buf[offset:offset + nnz] = torch.from_numpy(rows).to(cuda)
    row = buf[offset:offset + nnz]
    rp = torch.full((m + 1,), -7, dtype=torch.int32, device=cuda)
    stream = C.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    rc = sblas_lib.sblas_coo_rows_to_rowptr(m, nnz, C.c_void_p(row.data_ptr()),
                                            C.c_void_p(rp.data_ptr()), stream)
    assert rc == 0
    torch.cuda.synchronize()
    want = np.searchsorted(rows, np.arange(m + 1), side="left").astype(np.int32)
    np.testing.assert_array_equal(rp.cpu().numpy(), want)


@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_misaligned_device_arrays(sblas_lib, cuda, kernel):
    """Row pointer, columns and values as views 4 / 8 bytes past a 16-byte
    boundary: the tile kernel stages them with plain loads instead of bulk
    copies and partitions with the one-row-per-thread pass; results as for
    aligned arrays.  Power-law matrix of 200k rows, every tile shape."""
    from hpda_sblas_pnnl_gb300 import ops, synth
    a, x = synth.powerlaw(m=200_000, mean_deg=12.0, seed=77, values="normal")
    rp, col, val = a.numpy()

    def shifted(arr, dt):
        buf = torch.zeros(arr.size + 1, dtype=dt, device=cuda)
        buf[1:] = torch.from_numpy(np.ascontiguousarray(arr)).to(cuda)
        return buf[1:]

    d_rp, d_col, d_val = shifted(rp, torch.int32), shifted(col, torch.int32), shifted(val,
                                                                                   torch.float64)
    assert d_rp.data_ptr() % 16 != 0 and d_val.data_ptr() % 16 != 0
    xd = x.to(cuda)
    y0 = torch.randn(a.m, dtype=torch.float64, device=cuda)
    ref = O.csr_spmv(a.m, a.n, rp, col, val, x.numpy(), y0.cpu().numpy(), 1.5, -0.5)
    sig = sigmas() if kernel != 1 else [0]
    for s in sig:
        y = y0.clone()
        ops.csrmv(d_rp, d_col, d_val, xd, y, 1.5, -0.5, n=a.n, kernel=kernel, sigma=s)
        torch.cuda.synchronize()
        assert_close(y.cpu().numpy(), ref)
