"""The oracle (CPU restatement) pinned against the reference's own CPU code:
the golden fixtures were produced by the reference's functions compiled
from its sources (tests/golden/make_golden.py), and, where oracle/_ref is
built in this container, the oracle is also compared with them directly on
fresh random inputs."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden_cases, load_golden
from oracle import oracle as O


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_csr_matches_reference_golden(name):
    g = load_golden(name)
    y = O.csr_spmv(int(g["m"]), int(g["n"]), g["rowptr"], g["col"], g["val"], g["x"], g["y0"],
                   float(g["alpha"]), float(g["beta"]))
    np.testing.assert_array_equal(y, g["y_ref_csr"])   # bit-exact: same summation order


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_coo_matches_reference_golden(name):
    g = load_golden(name)
    y = O.coo_spmv(int(g["m"]), int(g["n"]), g["coo_row"], g["col"], g["val"], g["x"], g["y0"],
                   float(g["alpha"]), float(g["beta"]))
    np.testing.assert_array_equal(y, g["y_ref_coo"])


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_threaded_and_csc_forms(name):
    g = load_golden(name)
    m, n = int(g["m"]), int(g["n"])
    a, b = float(g["alpha"]), float(g["beta"])
    y = O.csr_spmv(m, n, g["rowptr"], g["col"], g["val"], g["x"], g["y0"], a, b, threads=4)
    np.testing.assert_array_equal(y, g["y_ref_csr"])    # per-row order kept
    yc = O.csc_spmv(m, n, g["csc_colptr"], g["csc_row"], g["csc_val"], g["x"], g["y0"], a, b)
    ref = g["y_ref_csr"]
    assert np.linalg.norm(yc - ref) <= 1e-13 * max(1.0, np.linalg.norm(ref))


def test_g_known_answer():
    """test/dspmv_test_smt.cu:176-232 with x = 1: y[i] = nnz of row i."""
    r, c, v = O.gen_g(200)
    assert r.size == 4850
    val, rowptr, col = O.coo2csr(200, 200, v, r, c)
    y = O.csr_spmv(200, 200, rowptr, col, val, np.ones(200), np.zeros(200))
    assert (y[:25] == 180).all() and (y[25:] == 2).all()
    with pytest.raises(ValueError):
        O.gen_g(201)   # the reference overruns rows when n % 8 != 0


def test_search_helpers_match_reference_golden():
    g = load_golden("search")
    a = g["a"]
    for k, f, l in zip(g["keys"], g["first"], g["last"]):
        assert O.find_first_in_sorted(a, a.size - 1, int(k)) == f
        assert O.find_last_in_sorted(a, a.size - 1, int(k)) == l
    rp = g["rowptr"]
    for i, r in zip(g["idx"], g["row_of"]):
        assert O.get_row_from_index(rp.size - 1, rp, int(i)) == r


def test_coo_conversions_match_scipy():
    rng = np.random.default_rng(7)
    m, n, nnz = 300, 250, 4000
    row = rng.integers(0, m, nnz).astype(np.int32)
    col = rng.integers(0, n, nnz).astype(np.int32)
    val = rng.normal(size=nnz)
    v, p, c = O.coo2csr(m, n, val, row, col)
    ref = sp.coo_matrix((val, (row, col)), shape=(m, n)).tocsr()
    ref.sum_duplicates()
    mine = sp.csr_matrix((v, c, p), shape=(m, n))
    assert abs(mine - ref).max() < 1e-12
    v2, p2, r2 = O.coo2csc(m, n, val, row, col)
    mine2 = sp.csc_matrix((v2, r2, p2), shape=(m, n))
    assert abs(mine2 - ref).max() < 1e-12


@pytest.mark.parametrize("nparts", [1, 2, 3, 5, 8, 13])
def test_nnz_split_merge_reproduces_unsplit(nparts):
    """src/dspmv_mgpu_v1.cu partition + merge: splitting nnz into parts and
    fixing up the rows cut by a split gives the unsplit product."""
    g = load_golden("zipf200_ab")
    m, n = int(g["m"]), int(g["n"])
    a, b = float(g["alpha"]), float(g["beta"])
    y = O.csr_spmv_nnz_split(m, n, g["rowptr"], g["col"], g["val"], g["x"], g["y0"], nparts, a, b)
    ref = g["y_ref_csr"]
    assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)


def test_dot2_is_more_accurate():
    rng = np.random.default_rng(3)
    m = n = 50
    rowptr = np.arange(0, 50 * 200 + 1, 200, dtype=np.int32)
    col = rng.integers(0, n, 50 * 200).astype(np.int32)
    val = rng.normal(size=col.size) * 1e8
    x = rng.normal(size=n)
    exact = np.array([float(sum(__import__("fractions").Fraction(v) * __import__("fractions").Fraction(x[c])
                                for v, c in zip(val[rowptr[i]:rowptr[i + 1]], col[rowptr[i]:rowptr[i + 1]])))
                      for i in range(m)])
    y1 = O.csr_spmv(m, n, rowptr, col, val, x, np.zeros(m))
    y2 = O.csr_spmv(m, n, rowptr, col, val, x, np.zeros(m), dot2=True)
    assert np.abs(y2 - exact).max() <= np.abs(y1 - exact).max()
    assert np.abs(y2 - exact).max() <= 1e-15 * np.abs(val).max() * np.abs(x).max()


@pytest.mark.skipif(not O.ref_available(), reason="oracle/_ref not built (no reference sources)")
def test_oracle_equals_reference_binary_on_random_inputs():
    rng = np.random.default_rng(11)
    for trial in range(5):
        m, n = int(rng.integers(1, 400)), int(rng.integers(1, 400))
        deg = rng.integers(0, 30, m)
        rowptr = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
        col = rng.integers(0, n, int(rowptr[-1])).astype(np.int32)
        val = rng.normal(size=col.size)
        x = rng.normal(size=n)
        y0 = rng.normal(size=m)
        a, b = float(rng.normal()), float(rng.normal())
        np.testing.assert_array_equal(O.csr_spmv(m, n, rowptr, col, val, x, y0, a, b),
                                      O.ref_csr_spmv(m, n, rowptr, col, val, x, y0, a, b))
        np.testing.assert_array_equal(
            O.csr_spmv(m, n, rowptr, col, val, x, y0, a, b, threads=3),
            O.ref_csr_spmv(m, n, rowptr, col, val, x, y0, a, b, threads=3))
        row = np.repeat(np.arange(m, dtype=np.int32), deg).astype(np.int32)
        np.testing.assert_array_equal(O.coo_spmv(m, n, row, col, val, x, y0, a, b),
                                      O.ref_coo_spmv(m, n, row, col, val, x, y0, a, b))
        for idx in range(0, int(rowptr[-1]), 7):
            assert O.get_row_from_index(m, rowptr, idx) == O.ref_get_row_from_index(m, rowptr, idx)


def test_oracle_spmm_and_adjoints_match_scipy():
    """The multi-right-hand-side and adjoint restatements (oracle_csr_spmm,
    oracle_csr_spmm_t, oracle_csr_sddmm) against scipy.sparse."""
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(4)
    a = sp.random(300, 200, density=0.05, format="csr", random_state=4)
    rp, c, v = a.indptr.astype(np.int32), a.indices.astype(np.int32), a.data
    for k in (1, 3, 8):
        x = rng.standard_normal((200, k))
        y0 = rng.standard_normal((300, k))
        y = O.csr_spmm(300, 200, rp, c, v, x, y0, -1.5, 0.25)
        np.testing.assert_allclose(y, -1.5 * (a @ x) + 0.25 * y0, rtol=1e-13, atol=1e-13)
        ypat = O.csr_spmm(300, 200, rp, c, None, x, y0, 1.0, 0.0)
        np.testing.assert_allclose(ypat, (a != 0).astype(np.float64) @ x, rtol=1e-13, atol=1e-13)
        g = rng.standard_normal((300, k))
        np.testing.assert_allclose(O.csr_spmm_t(300, 200, rp, c, v, g), a.T @ g, rtol=1e-13,
                                   atol=1e-13)
        rows = np.repeat(np.arange(300), np.diff(rp))
        np.testing.assert_allclose(O.csr_sddmm(300, 200, rp, c, g, x),
                                   np.einsum("pk,pk->p", g[rows], x[c]), rtol=1e-13, atol=1e-13)
    # one right-hand side as a 1-D vector is the plain SpMV loop, bit for bit
    x1 = rng.standard_normal(200)
    y1 = rng.standard_normal(300)
    np.testing.assert_array_equal(O.csr_spmm(300, 200, rp, c, v, x1, y1, 2.0, 0.5),
                                  O.csr_spmv(300, 200, rp, c, v, x1, y1, 2.0, 0.5))


def test_oracle_filter_x_matches_numpy_and_leaves_finite_products_unchanged():
    """spMspV's filter (src/dspmv_mgpu_v1.cu:29-40): kept nonzeros in storage
    order; with finite values the filtered product equals the unfiltered one
    bit for bit (the dropped terms are signed zeros added to a sum)."""
    rng = np.random.default_rng(12)
    a = sp.random(3000, 2000, density=0.01, format="csr", random_state=12)
    a.data = rng.standard_normal(a.nnz)
    rp, col, val = a.indptr.astype(np.int32), a.indices.astype(np.int32), a.data
    x = rng.uniform(-1, 1, 2000)
    x[rng.random(2000) < 0.7] = 0.0
    x[rng.random(2000) < 0.05] = -0.0
    orp, oc, ov = O.csr_filter_x(3000, rp, col, val, x)
    keep = x[col] != 0.0
    np.testing.assert_array_equal(oc, col[keep])
    np.testing.assert_array_equal(ov, val[keep])
    rows = np.repeat(np.arange(3000), np.diff(rp))
    np.testing.assert_array_equal(orp, np.concatenate([[0], np.cumsum(np.bincount(
        rows[keep], minlength=3000))]))
    full = O.csr_spmv(3000, 2000, rp, col, val, x, np.zeros(3000))
    filt = O.csr_spmv(3000, 2000, orp, oc, ov, x, np.zeros(3000))
    assert full.tobytes() == filt.tobytes()
