"""GPU parity of the batched SpMM (include/sblas_gb300.h, sblas_batch_*)
against the oracle's column-by-column restatement of the reference's CSR
loop (oracle_csr_spmm).  Tolerance: relative L2 <= 1e-12 per matrix and
right-hand side block, as for the single-matrix kernels."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL_L2 = 1e-12
EDGE_CASES = ["zipf200_ab", "long_row", "empty_rows", "sparse_rows", "diag3000", "g200", "one",
              "nnz0"]


def rel_l2(y, ref):
    den = np.linalg.norm(ref)
    num = np.linalg.norm(np.asarray(y) - ref)
    return num / den if den > 0 else num


def giant_row(cuda):
    """3 rows, the middle one 50 000 nonzeros long (crosses many units)."""
    rng = np.random.default_rng(9)
    rowptr = np.array([0, 2, 50_002, 50_005], dtype=np.int32)
    col = np.concatenate([[1, 7], np.sort(rng.choice(60_000, 50_000, replace=False)), [0, 3, 9]])
    val = rng.standard_normal(col.size)
    return (torch.from_numpy(rowptr).to(cuda), torch.from_numpy(col.astype(np.int32)).to(cuda),
            torch.from_numpy(val).to(cuda), 60_000)


def make_batch(cuda, seed=5):
    """Edge cases from the golden fixtures, a 50 000-nonzero row, an empty
    matrix and uneven synthetic matrices: list of (rowptr, col, val, n)."""
    from hpda_sblas_pnnl_gb300 import synth
    out = []
    for name in EDGE_CASES:
        g = load_golden(name)
        out.append((torch.from_numpy(g["rowptr"].astype(np.int32)).to(cuda),
                    torch.from_numpy(g["col"].astype(np.int32)).to(cuda),
                    torch.from_numpy(g["val"].astype(np.float64)).to(cuda), int(g["n"])))
    out.append(giant_row(cuda))
    out.append((torch.zeros(1, dtype=torch.int32, device=cuda),
                torch.zeros(0, dtype=torch.int32, device=cuda),
                torch.zeros(0, dtype=torch.float64, device=cuda), 4))       # m = 0
    for a in synth.batch_uneven(nmat=8, rows=(200, 20_000), deg=(2.0, 64.0), seed=seed,
                                device=cuda):
        out.append((a.rowptr, a.col, a.val, a.n))
    return out


def oracle_block(rp, col, val, n, x, y0, alpha, beta):
    m = rp.numel() - 1
    v = None if val is None else val.double().cpu().numpy()
    return O.csr_spmm(m, n, rp.cpu().numpy(), col.cpu().numpy(), v, x.cpu().numpy(),
                      y0.cpu().numpy(), alpha, beta)


def forms(val):
    return {"f64": val, "f32": val.float(), "pattern": None}


@pytest.mark.parametrize("k", [1, 2, 4, 8, 16])
@pytest.mark.parametrize("s", [4, 8, 16, 32])
def test_batch_matches_oracle(sblas_lib, cuda, k, s):
    from hpda_sblas_pnnl_gb300 import ops
    batch = make_batch(cuda)
    g = torch.Generator(device=cuda)
    g.manual_seed(100 * k + s)
    for form in ("f64", "f32", "pattern"):
        mats, xs, ys, y0s = [], [], [], []
        for rp, col, val, n in batch:
            m = rp.numel() - 1
            shape_x = (n, k) if k > 1 else (n,)
            shape_y = (m, k) if k > 1 else (m,)
            x = torch.rand(shape_x, generator=g, dtype=torch.float64, device=cuda) * 2 - 1
            y0 = torch.rand(shape_y, generator=g, dtype=torch.float64, device=cuda) * 2 - 1
            mats.append((rp, col, forms(val)[form]))
            xs.append(x)
            ys.append(y0.clone())
            y0s.append(y0)
        alpha, beta = 1.5, -0.25
        plan = ops.BatchPlan(mats, xs, ys, k, alpha=alpha, beta=beta, s=s)
        assert plan.s == s
        plan()
        torch.cuda.synchronize()
        for i, ((rp, col, v), x, y, y0) in enumerate(zip(mats, xs, ys, y0s)):
            ref = oracle_block(rp, col, v, x.shape[0], x, y0, alpha, beta)
            err = rel_l2(y.cpu().numpy(), ref)
            assert err <= RTOL_L2, (form, i, err)
        plan.close()


def test_batch_alpha1_beta0_never_reads_y(sblas_lib, cuda):
    """beta == 0: NaNs in Y are overwritten, not propagated."""
    from hpda_sblas_pnnl_gb300 import ops
    batch = make_batch(cuda)
    k = 4
    mats, xs, ys = [], [], []
    for rp, col, val, n in batch:
        mats.append((rp, col, val))
        xs.append(torch.rand((n, k), dtype=torch.float64, device=cuda))
        ys.append(torch.full((rp.numel() - 1, k), float("nan"), dtype=torch.float64, device=cuda))
    ops.BatchPlan(mats, xs, ys, k)()
    torch.cuda.synchronize()
    for (rp, col, v), x, y in zip(mats, xs, ys):
        ref = oracle_block(rp, col, v, x.shape[0], x, torch.zeros_like(y), 1.0, 0.0)
        assert np.isfinite(y.cpu().numpy()).all()
        assert rel_l2(y.cpu().numpy(), ref) <= RTOL_L2


def test_batch_graph_capture_replays_with_new_inputs(sblas_lib, cuda):
    """The run is graph-capturable: replays read the current contents of X."""
    from hpda_sblas_pnnl_gb300 import ops
    batch = make_batch(cuda, seed=6)
    k = 8
    mats = [(rp, col, val) for rp, col, val, _ in batch]
    xs = [torch.rand((n, k), dtype=torch.float64, device=cuda) for *_, n in batch]
    ys = [torch.zeros((rp.numel() - 1, k), dtype=torch.float64, device=cuda) for rp, *_ in batch]
    plan = ops.BatchPlan(mats, xs, ys, k)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan()
    torch.cuda.current_stream().wait_stream(s)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        plan()
    for rep in range(2):
        for x in xs:
            x.uniform_(-1, 1)
        graph.replay()
        torch.cuda.synchronize()
        for (rp, col, v), x, y in zip(mats, xs, ys):
            ref = oracle_block(rp, col, v, x.shape[0], x, torch.zeros_like(y), 1.0, 0.0)
            assert rel_l2(y.cpu().numpy(), ref) <= RTOL_L2


@pytest.mark.parametrize("k,split16", [(1, True), (8, False), (16, True), (16, False)])
def test_single_matrix_plan_takes_x_y_per_call(sblas_lib, cuda, k, split16):
    """k = 16 plans run as one pass by default, as two k = 8 passes with split16."""
    from hpda_sblas_pnnl_gb300 import ops, synth
    a, _ = synth.powerlaw(m=30_000, mean_deg=20.0, seed=11, device=cuda, values="normal")
    plan = ops.SpmmPlan(a.rowptr, a.col, a.val, n=a.n, k=k, split16=split16)
    for alpha, beta in ((1.0, 0.0), (3.0, 0.0), (-2.0, 0.5)):
        shape_x = (a.n, k) if k > 1 else (a.n,)
        shape_y = (a.m, k) if k > 1 else (a.m,)
        x = torch.randn(shape_x, dtype=torch.float64, device=cuda)
        y0 = torch.randn(shape_y, dtype=torch.float64, device=cuda)
        y = y0.clone()
        plan(x, y, alpha, beta)
        torch.cuda.synchronize()
        ref = oracle_block(a.rowptr, a.col, a.val, a.n, x, y0, alpha, beta)
        assert rel_l2(y.cpu().numpy(), ref) <= RTOL_L2
        y2 = y0.clone()                         # the same bits on a second run
        plan(x, y2, alpha, beta)
        assert torch.equal(y, y2)


def test_batch_rejects_misaligned_x(sblas_lib, cuda):
    from hpda_sblas_pnnl_gb300 import _lib, ops
    rp = torch.tensor([0, 1], dtype=torch.int32, device=cuda)
    col = torch.tensor([0], dtype=torch.int32, device=cuda)
    val = torch.ones(1, dtype=torch.float64, device=cuda)
    buf = torch.zeros(9, dtype=torch.float64, device=cuda)
    x = buf[1:5].view(2, 2)            # 8-byte offset: not 16-byte aligned
    y = torch.zeros((1, 2), dtype=torch.float64, device=cuda)
    with pytest.raises(_lib.SblasError):
        ops.BatchPlan([(rp, col, val)], [x], [y], 2)


@pytest.mark.parametrize("k", [1, 8])
def test_row_ids_write_listed_rows_only(sblas_lib, cuda, k):
    """A matrix stored without its empty rows (row_ids lists the rows of Y
    that stored rows write): listed rows equal the full product, unlisted
    rows keep their contents."""
    from hpda_sblas_pnnl_gb300 import ops
    g = load_golden("empty_rows")
    rp = g["rowptr"].astype(np.int64)
    m, n = int(g["m"]), int(g["n"])
    keep = np.nonzero(rp[1:] > rp[:-1])[0]
    rp_c = np.concatenate([rp[keep], rp[-1:]]).astype(np.int32)
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(device=cuda, dtype=dt)
    x = torch.rand((n, k) if k > 1 else (n,), dtype=torch.float64, device=cuda)
    y0 = torch.full((m, k) if k > 1 else (m,), 7.0, dtype=torch.float64, device=cuda)
    y = y0.clone()
    mat = (t(rp_c, torch.int32), t(g["col"], torch.int32), t(g["val"], torch.float64),
           t(keep, torch.int32))
    plan = ops.BatchPlan([mat], [x], [y], k, alpha=2.0, beta=0.5)
    plan()
    torch.cuda.synchronize()
    full = O.csr_spmm(m, n, g["rowptr"].astype(np.int32), g["col"].astype(np.int32),
                      g["val"].astype(np.float64), x.cpu().numpy(), y0.cpu().numpy(), 2.0, 0.5)
    yy = y.cpu().numpy()
    assert rel_l2(yy[keep], full[keep]) <= RTOL_L2
    rest = np.setdiff1d(np.arange(m), keep)
    assert (yy[rest] == 7.0).all()


@pytest.mark.parametrize("k", [8, 16])
@pytest.mark.parametrize("s", [4, 8])
def test_row_lengths_at_group_and_unit_boundaries(sblas_lib, cuda, k, s):
    """The k >= 8 kernel splits each unit of 32*s nonzeros into 32/k groups
    of k*s: rows of exactly one group, one more or one less, rows that fill
    a unit or cross several, empty rows between them and at the ends, in
    every order.  Within 1e-12 of the oracle; the same bits on a rerun."""
    from hpda_sblas_pnnl_gb300 import ops
    h, unit = k * s, 32 * s
    lengths = [0, 1, h - 1, h, h + 1, 2 * h, unit, unit + 1, 3 * unit + 7, 2, 0, 0]
    rng = np.random.default_rng(1000 * k + s)
    deg = np.array([lengths[i] for i in rng.integers(0, len(lengths), 400)] + [0, 0])
    deg = np.concatenate([[0], deg])
    m, n = deg.size, 5000
    rp = np.zeros(m + 1, np.int32)
    rp[1:] = np.cumsum(deg)
    col = np.concatenate([np.sort(rng.choice(n, size=d, replace=False)) for d in deg]).astype(np.int32)
    val = rng.standard_normal(col.size)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    x = torch.rand((n, k), dtype=torch.float64, device=cuda) * 2 - 1
    y0 = torch.rand((m, k), dtype=torch.float64, device=cuda) * 2 - 1
    for alpha, beta in ((1.0, 0.0), (0.5, 0.0), (1.5, -0.25)):
        plan = ops.SpmmPlan(t(rp), t(col), t(val), n=n, k=k, s=s)
        y = y0.clone()
        plan(x, y, alpha, beta)
        y2 = y0.clone()
        plan(x, y2, alpha, beta)
        torch.cuda.synchronize()
        ref = O.csr_spmm(m, n, rp, col, val, x.cpu().numpy(), y0.cpu().numpy(), alpha, beta)
        assert rel_l2(y.cpu().numpy(), ref) <= RTOL_L2, (alpha, beta)
        assert torch.equal(y, y2)
        plan.close()
