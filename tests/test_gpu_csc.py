"""CSC SpMV and the library's own sorts, on the GPU, against the oracle.

sblas_dcscmv (the device form of spMV_mgpu_baseline_csc,
src/dspmv_mgpu_baseline_csc.cu:131-135) is an inspector (a stable least-
significant-digit bucket sort of the entries by row: A's row-ordered
structure and the permutation to it) and an executor (the values gathered
into row order, then the CSR tile kernel).  Checked here: the golden
fixtures (the reference's own CPU loop), random matrices with empty and very
long columns, unsorted rows inside columns, row counts needing two and three
digit passes, alpha/beta, NaN in y with beta = 0, run-to-run bit equality,
the analysed plan reused with new values and with values bound once, and
the plan's staged value move (patterns of several 2^22-entry buckets) bit
for bit against the one-shot product's direct gather.  The conversions (CSC -> CSR,
A -> A^T with its permutation) are compared with numpy's stable sort
exactly.
"""
import numpy as np
import pytest
import torch

from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _rel(y, ref):
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(y - ref) / (den if den > 0 else 1.0))


def _csc_from_coo(m, n, rows, cols, vals):
    """CSC arrays, rows ascending inside each column (numpy stable sort)."""
    order = np.lexsort((rows, cols))
    colptr = np.zeros(n + 1, np.int32)
    np.add.at(colptr, cols + 1, 1)
    colptr = np.cumsum(colptr).astype(np.int32)
    return colptr, rows[order].astype(np.int32), vals[order]


def _random_csc(rng, m, n, nnz, long_col=None):
    rows = rng.integers(0, m, nnz)
    cols = rng.integers(0, n, nnz)
    if long_col is not None:
        k = min(nnz // 3, m)
        cols[:k] = long_col
        rows[:k] = rng.choice(m, k, replace=False)
    key = np.unique(cols.astype(np.int64) * m + rows)
    rows, cols = (key % m).astype(np.int32), (key // m).astype(np.int32)
    vals = rng.standard_normal(rows.size)
    return _csc_from_coo(m, n, rows, cols, vals)


def _dev(cuda, *arrays):
    return [torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in arrays]


@pytest.mark.parametrize("name", golden_cases())
def test_cscmv_golden(sblas_lib, cuda, name):
    from hpda_sblas_pnnl_gb300 import ops
    g = load_golden(name)
    m, n = int(g["m"]), int(g["n"])
    cp, ri, cv, x, y0 = _dev(cuda, g["csc_colptr"], g["csc_row"], g["csc_val"], g["x"], g["y0"])
    y = y0.clone()
    ops.cscmv(cp, ri, cv, x, y, float(g["alpha"]), float(g["beta"]))
    assert _rel(y.cpu().numpy(), g["y_ref_csr"]) <= TOL


@pytest.mark.parametrize("m,n,nnz,long_col", [
    (1, 50, 40, None),
    (7, 9, 30, None),
    (2048, 3000, 40_000, 5),
    (2049, 100, 30_000, None),           # m just past a power of two
    (100_000, 80_000, 1_500_000, 17),    # a column of 500k entries
    (4_200_000, 4_000_000, 3_000_000, None),   # three digit passes
    (9_000_000, 2_000_000, 1_200_000, None),
])
def test_cscmv_random_against_oracle(sblas_lib, cuda, m, n, nnz, long_col):
    from hpda_sblas_pnnl_gb300 import ops
    from oracle import oracle as O
    rng = np.random.default_rng(m + nnz)
    colptr, rowidx, val = _random_csc(rng, m, n, nnz, long_col)
    x = rng.standard_normal(n)
    y0 = rng.standard_normal(m)
    cp, ri, cv, xd = _dev(cuda, colptr, rowidx, val, x)
    for alpha, beta in ((1.0, 0.0), (-0.75, 0.0), (1.5, -0.5)):
        ref = O.csc_spmv(m, n, colptr, rowidx, val, x, y0, alpha, beta)
        yd = torch.from_numpy(y0.copy()).to(cuda)
        if beta == 0.0:
            yd.fill_(float("nan"))       # beta = 0 never reads y
        ops.cscmv(cp, ri, cv, xd, yd, alpha, beta)
        assert _rel(yd.cpu().numpy(), ref) <= TOL, (alpha, beta)
    # bit for bit the same on a second run, and through an analysed plan
    y1 = torch.zeros(m, dtype=torch.float64, device=cuda)
    y2 = torch.zeros(m, dtype=torch.float64, device=cuda)
    ops.cscmv(cp, ri, cv, xd, y1)
    ops.cscmv(cp, ri, cv, xd, y2)
    assert torch.equal(y1, y2)
    plan = ops.CscPlan(m, cp, ri)
    plan(cv, xd, y2)
    assert torch.equal(y1, y2)
    cv2 = cv * -2.0                                    # new values, same pattern
    plan(cv2, xd, y2, 0.5, 0.0)
    ref = O.csc_spmv(m, n, colptr, rowidx, -2.0 * val, x, np.zeros(m), 0.5, 0.0)
    assert _rel(y2.cpu().numpy(), ref) <= TOL
    # values bound once (kept in row order): calls without values, same bits
    plan.bind(cv)
    y3 = torch.zeros(m, dtype=torch.float64, device=cuda)
    plan(None, xd, y3)
    assert torch.equal(y1, y3)


def test_cscmv_unsorted_rows_and_empty(sblas_lib, cuda):
    """Rows in any order inside a column, empty leading/trailing columns and
    rows, nnz = 0."""
    from hpda_sblas_pnnl_gb300 import ops
    from oracle import oracle as O
    rng = np.random.default_rng(5)
    m, n = 5000, 700
    colptr, rowidx, val = _random_csc(rng, m, n, 20_000)
    colptr[:20] = 0                                   # empty leading columns
    colptr[-30:] = colptr[-31]                        # empty trailing columns
    nnz = int(colptr[-1])
    rowidx, val = rowidx[:nnz].copy(), val[:nnz].copy()
    for j in range(n):                                # shuffle rows inside columns
        s = slice(colptr[j], colptr[j + 1])
        p = rng.permutation(colptr[j + 1] - colptr[j])
        rowidx[s], val[s] = rowidx[s][p], val[s][p]
    x = rng.standard_normal(n)
    ref = O.csc_spmv(m, n, colptr, rowidx, val, x, np.zeros(m))
    cp, ri, cv, xd = _dev(cuda, colptr, rowidx, val, x)
    y = torch.zeros(m, dtype=torch.float64, device=cuda)
    ops.cscmv(cp, ri, cv, xd, y)
    assert _rel(y.cpu().numpy(), ref) <= TOL
    # no entries at all: y = beta * y
    cp0 = torch.zeros(n + 1, dtype=torch.int32, device=cuda)
    e = torch.zeros(0, dtype=torch.int32, device=cuda)
    ev = torch.zeros(0, dtype=torch.float64, device=cuda)
    y = torch.full((m,), 3.0, dtype=torch.float64, device=cuda)
    ops.cscmv(cp0, e, ev, xd, y, 1.0, 0.5)
    assert torch.equal(y, torch.full_like(y, 1.5))


@pytest.mark.parametrize("m,n,nnz", [(300, 200, 5000), (3_000_000, 2_500_000, 4_000_000),
                                     (9_000_000, 100_000, 800_000)])
def test_csc_to_csr_and_transpose_match_stable_sort(sblas_lib, cuda, m, n, nnz):
    """Own LSD bucket sort, 8-bit digits: two passes for keys below 2^16,
    three up to 2^24."""
    from hpda_sblas_pnnl_gb300 import ops
    rng = np.random.default_rng(nnz)
    colptr, rowidx, val = _random_csc(rng, m, n, nnz)
    cols = np.repeat(np.arange(n, dtype=np.int32), np.diff(colptr))
    order = np.argsort(rowidx, kind="stable")         # CSC order -> CSR order
    want_rp = np.zeros(m + 1, np.int64)
    np.add.at(want_rp, rowidx.astype(np.int64) + 1, 1)
    want_rp = np.cumsum(want_rp)
    cp, ri, cv = _dev(cuda, colptr, rowidx, val)
    rp, c, v = ops.csc_to_csr(m, n, cp, ri, cv)
    np.testing.assert_array_equal(rp.cpu().numpy(), want_rp)
    np.testing.assert_array_equal(c.cpu().numpy(), cols[order])
    assert v.cpu().numpy().tobytes() == val[order].tobytes()
    # A^T of that CSR matrix is the CSC form again, with the permutation
    t_rp, t_c, perm = ops.csr_transpose(m, n, rp, c)
    np.testing.assert_array_equal(t_rp.cpu().numpy(), colptr)
    np.testing.assert_array_equal(t_c.cpu().numpy(), rowidx)
    back = np.argsort(order, kind="stable")           # CSC position -> CSR position
    np.testing.assert_array_equal(perm.cpu().numpy(), back)


@pytest.mark.parametrize("m,n,nnz,long_col", [
    (3_000_000, 2_000_000, 9_000_000, None),       # 3 staging buckets of 2^22 entries
    (6_000_000, 5_000_000, 17_500_000, 123),       # 5 buckets (8 digit values), a long column
])
def test_csc_plan_staged_matches_direct_bit_for_bit(sblas_lib, cuda, m, n, nnz, long_col):
    """An analysed plan above one 2^22-entry bucket moves values through the
    staging array (a streaming scatter into per-bucket runs, then a gather
    inside each bucket); the one-shot product gathers them directly.  Both
    feed the same tile kernel the same row-ordered values: equal bits, and
    the oracle within 1e-12."""
    from hpda_sblas_pnnl_gb300 import ops
    from oracle import oracle as O
    rng = np.random.default_rng(nnz)
    colptr, rowidx, val = _random_csc(rng, m, n, nnz, long_col)
    x = rng.standard_normal(n)
    y0 = rng.standard_normal(m)
    cp, ri, cv, xd, y0d = _dev(cuda, colptr, rowidx, val, x, y0)
    direct = y0d.clone()
    ops.cscmv(cp, ri, cv, xd, direct, 0.5, -1.25)
    plan = ops.CscPlan(m, cp, ri)
    staged = y0d.clone()
    plan(cv, xd, staged, 0.5, -1.25)
    assert torch.equal(staged, direct)
    ref = O.csc_spmv(m, n, colptr, rowidx, val, x, y0, 0.5, -1.25)
    assert _rel(staged.cpu().numpy(), ref) <= TOL
    cv2 = torch.flip(cv, [0]).contiguous()               # new values through the plan
    plan(cv2, xd, staged)
    direct.zero_()
    ops.cscmv(cp, ri, cv2, xd, direct)
    assert torch.equal(staged, direct)
    plan.bind(cv)                                        # bound values: staged once
    y3 = y0d.clone()
    plan(None, xd, y3, 0.5, -1.25)
    y4 = y0d.clone()
    ops.cscmv(cp, ri, cv, xd, y4, 0.5, -1.25)
    assert torch.equal(y3, y4)


@pytest.mark.parametrize("m,n,nnz", [
    (1500, 4000, 1 << 20),            # exactly one bucket: the plan keeps the direct gather
    (1500, 4000, (1 << 20) + 1),      # a second bucket holding one entry
    (3, 1_500_000, (1 << 21) + 7),    # three rows, each spanning buckets
    (700_000, 5, (1 << 21) + 7),      # five columns, each spanning buckets
])
def test_csc_plan_staging_bucket_edges(sblas_lib, cuda, m, n, nnz):
    """Exact entry counts at the 2^20-entry staging bucket boundaries, and
    rows and columns far longer than a bucket: the plan's staged values
    equal the one-shot product's direct gather bit for bit."""
    from hpda_sblas_pnnl_gb300 import ops
    from oracle import oracle as O
    rng = np.random.default_rng(nnz + m)
    key = np.sort(rng.choice(m * n, size=nnz, replace=False))
    rows, cols = (key % m).astype(np.int64), (key // m).astype(np.int64)
    colptr, rowidx, val = _csc_from_coo(m, n, rows, cols, rng.standard_normal(nnz))
    assert rowidx.size == nnz
    x = rng.standard_normal(n)
    cp, ri, cv, xd = _dev(cuda, colptr, rowidx, val, x)
    direct = torch.zeros(m, dtype=torch.float64, device=cuda)
    ops.cscmv(cp, ri, cv, xd, direct)
    plan = ops.CscPlan(m, cp, ri)
    staged = torch.full((m,), float("nan"), dtype=torch.float64, device=cuda)
    plan(cv, xd, staged)
    assert torch.equal(staged, direct)
    ref = O.csc_spmv(m, n, colptr, rowidx, val, x, np.zeros(m))
    assert _rel(staged.cpu().numpy(), ref) <= TOL


@pytest.mark.parametrize("case", ["one_entry", "one_row", "one_column", "every_row_once"])
def test_sort_edge_cases(sblas_lib, cuda, case):
    """The bucket sort on degenerate key sets: a single entry, every key
    equal (all entries in one row: stability alone orders them), one dense
    column, a permutation matrix (every key once)."""
    from hpda_sblas_pnnl_gb300 import ops
    from oracle import oracle as O
    rng = np.random.default_rng(11)
    if case == "one_entry":
        m, n, rows, cols = 5_000_000, 3, np.array([4_999_999]), np.array([1])
    elif case == "one_row":
        m, n = 3_000_000, 50_000
        cols = np.arange(n)
        rows = np.full(n, 2_999_998)
    elif case == "one_column":
        m, n = 70_000, 9
        rows = np.arange(m)
        cols = np.full(m, 4)
    else:
        m = n = 300_000
        rows = rng.permutation(m)
        cols = np.arange(n)
    vals = rng.standard_normal(rows.size)
    colptr, rowidx, val = _csc_from_coo(m, n, rows.astype(np.int64), cols.astype(np.int64), vals)
    x = rng.standard_normal(n)
    cp, ri, cv, xd = _dev(cuda, colptr, rowidx, val, x)
    rp, c, v = ops.csc_to_csr(m, n, cp, ri, cv)
    order = np.argsort(rowidx, kind="stable")
    ccols = np.repeat(np.arange(n, dtype=np.int32), np.diff(colptr))
    np.testing.assert_array_equal(c.cpu().numpy(), ccols[order])
    assert v.cpu().numpy().tobytes() == val[order].tobytes()
    assert int(rp[-1]) == rows.size and int(rp[0]) == 0
    y = torch.zeros(m, dtype=torch.float64, device=cuda)
    ops.cscmv(cp, ri, cv, xd, y)
    ref = O.csc_spmv(m, n, colptr, rowidx, val, x, np.zeros(m))
    assert _rel(y.cpu().numpy(), ref) <= TOL
