"""Seeded synthetic matrices (CPU): structure and reproducibility."""
import torch

from hpda_sblas_pnnl_gb300 import synth


def _rows(a):
    return torch.repeat_interleave(torch.arange(a.m), (a.rowptr[1:] - a.rowptr[:-1]).long())


def test_row_sums_fixed_order():
    rp = torch.tensor([0, 2, 2, 5, 5], dtype=torch.int32)
    v = torch.arange(5, dtype=torch.float64) + 1
    want = torch.tensor([3.0, 0.0, 12.0, 0.0], dtype=torch.float64)
    for chunk in (1, 2, 3, 1 << 16):
        assert torch.equal(synth._row_sums(rp, v, rows_per_chunk=chunk), want)
    assert synth._row_sums(torch.zeros(1, dtype=torch.int32), torch.zeros(0, dtype=torch.float64)).numel() == 0


def test_banded_fem_diagonally_dominant_and_reproducible():
    a, x = synth.banded_fem(m=9_001, per_row=20, band=600, seed=5)
    b, y = synth.banded_fem(m=9_001, per_row=20, band=600, seed=5)
    assert torch.equal(a.rowptr, b.rowptr) and torch.equal(a.col, b.col)
    assert torch.equal(a.val, b.val) and torch.equal(x, y)
    r = _rows(a)
    diag = a.col.long() == r
    assert int(diag.sum()) == a.m                      # every row holds its diagonal
    off = torch.zeros(a.m, dtype=torch.float64).index_add_(
        0, r, torch.where(diag, 0.0, a.val.abs()))
    torch.testing.assert_close(a.val[diag], 1.0 + off, rtol=1e-14, atol=0)
    assert bool((a.col[1:] > a.col[:-1])[(r[1:] == r[:-1])].all())   # sorted, no duplicates


def test_powerlaw_shape():
    a, x = synth.powerlaw(m=5_000, mean_deg=8.0, dmax=500, seed=7)
    assert a.rowptr.numel() == 5_001 and int(a.rowptr[-1]) == a.nnz
    assert int((a.rowptr[1:] - a.rowptr[:-1]).min()) >= 1
    assert int(a.col.min()) >= 0 and int(a.col.max()) < a.n and x.numel() == a.n
