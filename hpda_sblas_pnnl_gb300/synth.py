"""Seeded synthetic sparse matrices standing in for the reference's inputs.

The reference measures on SuiteSparse power-law graphs and FEM matrices
(data/download_matrix_power_law.sh) that are not available here; these
generators produce matrices of the shapes, sizes and value distributions of
the benchmark configurations instead.  All run on torch (CPU or CUDA) and
return CSR with int32 indices, columns sorted and unique inside each row.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch


@dataclass
class CSR:
    m: int
    n: int
    rowptr: torch.Tensor  # int32 [m + 1]
    col: torch.Tensor     # int32 [nnz]
    val: torch.Tensor     # float64 [nnz]

    @property
    def nnz(self) -> int:
        return int(self.col.numel())

    def to(self, device) -> "CSR":
        return CSR(self.m, self.n, self.rowptr.to(device), self.col.to(device),
                   self.val.to(device))

    def numpy(self):
        return (self.rowptr.cpu().numpy(), self.col.cpu().numpy(), self.val.cpu().numpy())


def _gen(seed: int, device) -> torch.Generator:
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    return g


def _csr_from_keys(m: int, n: int, rows: torch.Tensor, cols: torch.Tensor,
                   dedupe: bool = True) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Sorts (row, col) pairs, removes duplicates; returns rowptr, col, perm."""
    key = rows.to(torch.int64) * n + cols.to(torch.int64)
    key, perm = torch.sort(key, stable=True)
    if dedupe:
        keep = torch.ones_like(key, dtype=torch.bool)
        keep[1:] = key[1:] != key[:-1]
        key = key[keep]
        perm = perm[keep]
    r = torch.div(key, n, rounding_mode="floor")
    c = (key - r * n).to(torch.int32)
    counts = torch.bincount(r, minlength=m)
    rowptr = torch.zeros(m + 1, dtype=torch.int64, device=key.device)
    rowptr[1:] = torch.cumsum(counts, 0)
    return rowptr.to(torch.int32), c, perm


def zipf_rows(n: int = 200, s: float = 1.5, seed: int = 200, device="cpu") -> tuple[CSR, torch.Tensor]:
    """Square n x n, per-row nnz ~ Zipf(s) clipped to [1, n], columns uniform
    without replacement, values and x ~ U(-1, 1) (the 'g'-mode stand-in)."""
    g = _gen(seed, device)
    # Zipf(s) by inverse transform on the truncated support 1..n
    k = torch.arange(1, n + 1, dtype=torch.float64, device=device)
    pmf = k.pow(-s)
    cdf = torch.cumsum(pmf / pmf.sum(), 0)
    u = torch.rand(n, generator=g, dtype=torch.float64, device=device)
    deg = torch.searchsorted(cdf, u).clamp(max=n - 1) + 1
    rows, cols = [], []
    for i in range(n):
        p = torch.randperm(n, generator=g, device=device)[: int(deg[i])]
        rows.append(torch.full((p.numel(),), i, dtype=torch.int64, device=device))
        cols.append(p)
    rowptr, col, _ = _csr_from_keys(n, n, torch.cat(rows), torch.cat(cols))
    val = torch.rand(col.numel(), generator=g, dtype=torch.float64, device=device) * 2 - 1
    x = torch.rand(n, generator=g, dtype=torch.float64, device=device) * 2 - 1
    return CSR(n, n, rowptr, col, val), x


def _pareto_xmin(alpha: float, dmax: int, mean: float) -> float:
    """xmin of floor(xmin * U^(-1/(alpha-1))) clipped to [1, dmax] with the
    requested mean (bisection on the closed-form continuous mean)."""
    a = alpha - 1.0

    def m(xmin: float) -> float:
        # E[min(X, dmax)] for X ~ Pareto(xmin, a), minus ~0.5 for the floor
        if xmin >= dmax:
            return dmax
        body = xmin * a / (a - 1.0) * (1.0 - (xmin / dmax) ** (a - 1.0)) if a != 1 else 0.0
        tail = dmax * (xmin / dmax) ** a
        return body + tail - 0.5

    lo, hi = 1.0, float(dmax)
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if m(mid) < mean:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def powerlaw(m: int = 4_000_000, mean_deg: float = 19.1, alpha: float = 2.1, dmax: int = 20_000,
             seed: int = 2021, device="cpu", values: str = "ones") -> tuple[CSR, torch.Tensor]:
    """Power-law graph (m x m): out-degrees ~ discrete Pareto with exponent
    alpha clipped to [1, dmax], scaled to mean_deg; endpoints by a
    preferential-attachment stand-in (Zipf popularity over randomly permuted
    column ids, exponent 1/(alpha-1), which gives power-law in-degrees).
    Duplicate endpoints are merged, so the stored nonzeros fall short of
    m * mean_deg: at m = 4M the default mean_deg of 19.1 draws ~76M and keeps
    ~70M (the benchmark size).
    values='ones' (binary pattern, 1.0) or 'normal' (N(0, 1)); x ~ U(0, 1)."""
    g = _gen(seed, device)
    xmin = _pareto_xmin(alpha, dmax, mean_deg)
    u = torch.rand(m, generator=g, dtype=torch.float64, device=device)
    deg = torch.floor(xmin * u.pow(-1.0 / (alpha - 1.0))).clamp_(1, dmax).to(torch.int64)
    total = int(deg.sum())
    rows = torch.repeat_interleave(torch.arange(m, device=device), deg)
    s = 1.0 / (alpha - 1.0)
    e = 1.0 - s
    uc = torch.rand(total, generator=g, dtype=torch.float64, device=device)
    rank = (((m + 1.0) ** e - 1.0) * uc + 1.0).pow(1.0 / e) - 1.0
    rank = rank.floor().clamp_(0, m - 1).to(torch.int64)
    perm = torch.randperm(m, generator=g, device=device)
    cols = perm[rank]
    del uc, rank
    rowptr, col, _ = _csr_from_keys(m, m, rows, cols)
    del rows, cols
    if values == "ones":
        val = torch.ones(col.numel(), dtype=torch.float64, device=device)
    else:
        val = torch.randn(col.numel(), generator=g, dtype=torch.float64, device=device)
    x = torch.rand(m, generator=g, dtype=torch.float64, device=device)
    return CSR(m, m, rowptr, col, val), x


def _row_sums(rowptr: torch.Tensor, v: torch.Tensor, rows_per_chunk: int = 1 << 16) -> torch.Tensor:
    """Sum of v over each CSR row, as a padded per-row reduction over chunks of
    rows: the summation order is fixed, so the sums are the same on every run
    (a scatter-add on the GPU accumulates in whatever order its atomics land)."""
    m = rowptr.numel() - 1
    out = torch.zeros(m, dtype=v.dtype, device=v.device)
    if m == 0 or v.numel() == 0:
        return out
    start = rowptr.to(torch.int64)
    lens = start[1:] - start[:-1]
    for r0 in range(0, m, rows_per_chunk):
        r1 = min(m, r0 + rows_per_chunk)
        ln = lens[r0:r1]
        j = torch.arange(int(ln.max()), device=v.device)
        ok = j[None, :] < ln[:, None]
        idx = (start[r0:r1, None] + j[None, :]).clamp_(max=v.numel() - 1)
        out[r0:r1] = torch.where(ok, v[idx], torch.zeros((), dtype=v.dtype, device=v.device)).sum(1)
    return out


def banded_fem(m: int = 2_000_000, per_row: int = 140, band: int = 20_000, offband: float = 0.01,
               seed: int = 3, device="cpu") -> tuple[CSR, torch.Tensor]:
    """FEM-like banded matrix: 3x3 dense blocks at random block columns within
    a band of total width `band` around the diagonal (the diagonal block
    always present), plus `offband` x per_row random entries per row anywhere.
    Values ~ N(0, 1), diagonal set to 1 + sum of |off-diagonal| of its row
    (diagonally dominant), x ~ N(0, 1)."""
    g = _gen(seed, device)
    nb = (m + 2) // 3  # the last block row may be partial
    half = band // 6  # block columns on each side of the diagonal block
    bpr = max(1, round(per_row * (1 - offband) / 3))  # blocks per block row
    br = torch.arange(nb, device=device).repeat_interleave(bpr)
    off = torch.randint(-half, half + 1, (nb * bpr,), generator=g, device=device)
    off.view(nb, bpr)[:, 0] = 0
    bc = (br + off).clamp_(0, nb - 1)
    # expand blocks to 3x3 entries
    a = torch.arange(3, device=device)
    rows = (3 * br[:, None, None] + a[None, :, None]).expand(-1, 3, 3).reshape(-1)
    cols = (3 * bc[:, None, None] + a[None, None, :]).expand(-1, 3, 3).reshape(-1)
    del br, off, bc
    if m % 3:
        keep = (rows < m) & (cols < m)
        rows, cols = rows[keep], cols[keep]
    n_off = int(round(per_row * offband * m))
    if n_off > 0:
        ro = torch.randint(0, m, (n_off,), generator=g, device=device)
        co = torch.randint(0, m, (n_off,), generator=g, device=device)
        rows = torch.cat([rows, ro])
        cols = torch.cat([cols, co])
    rowptr, col, _ = _csr_from_keys(m, m, rows, cols)
    del rows, cols
    val = torch.randn(col.numel(), generator=g, dtype=torch.float64, device=device)
    r = torch.repeat_interleave(torch.arange(m, device=device),
                                (rowptr[1:] - rowptr[:-1]).to(torch.int64))
    diag = col.to(torch.int64) == r
    absrow = _row_sums(rowptr, torch.where(diag, torch.zeros_like(val), val.abs()))
    val = torch.where(diag, 1.0 + absrow[r], val)
    x = torch.randn(m, generator=g, dtype=torch.float64, device=device)
    return CSR(m, m, rowptr, col, val), x


def batch_uneven(nmat: int = 64, rows: tuple[int, int] = (10_000, 1_000_000),
                 deg: tuple[float, float] = (4.0, 64.0), seed: int = 64,
                 device="cpu") -> list[CSR]:
    """Uneven batch: row counts log-uniform in `rows`, mean nonzeros per row
    log-uniform in `deg`; even-numbered matrices power-law (N(0, 1) values,
    maximum row length min(20000, m)), odd-numbered banded FEM-like (band
    width min(20000, m)).  Square matrices, FP64 values."""
    g = _gen(seed, "cpu")
    lo_r, hi_r = math.log(rows[0]), math.log(rows[1])
    lo_d, hi_d = math.log(deg[0]), math.log(deg[1])
    out = []
    for i in range(nmat):
        u = torch.rand(2, generator=g, dtype=torch.float64)
        m = int(round(math.exp(lo_r + (hi_r - lo_r) * float(u[0]))))
        d = math.exp(lo_d + (hi_d - lo_d) * float(u[1]))
        if i % 2 == 0:
            a, _ = powerlaw(m=m, mean_deg=d, dmax=min(20_000, m), seed=seed * 1000 + i,
                            device=device, values="normal")
        else:
            a, _ = banded_fem(m=m, per_row=max(3, int(round(d))), band=min(20_000, m),
                              seed=seed * 1000 + i, device=device)
        out.append(a)
    return out


def csr_to_coo_rows(a: CSR) -> torch.Tensor:
    """Row index of every nonzero (row-sorted COO)."""
    cnt = (a.rowptr[1:] - a.rowptr[:-1]).to(torch.int64)
    return torch.repeat_interleave(torch.arange(a.m, device=a.rowptr.device, dtype=torch.int32), cnt)


def csr_to_csc(a: CSR) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """Column-compressed copy (colptr, rowidx, val), rows ascending in each column."""
    rows = csr_to_coo_rows(a)
    colptr, rowidx, perm = _csr_from_keys(a.n, a.m, a.col, rows, dedupe=False)
    return colptr, rowidx, a.val[perm]


def compulsory_bytes(m: int, n: int, nnz: int, val_bytes: int = 8, beta_nonzero: bool = False,
                     fmt: str = "csr", k: int = 1) -> int:
    """Each array touched once: values, indices, row pointer, x read once,
    y written once (and read once if beta != 0), k right-hand sides."""
    if fmt == "coo":
        idx = 8 * nnz
    elif fmt == "csc":
        idx = 4 * nnz + 4 * (n + 1)
    else:
        idx = 4 * nnz + 4 * (m + 1)
    return val_bytes * nnz + idx + k * 8 * n + k * 8 * m * (2 if beta_nonzero else 1)


__all__ = ["CSR", "zipf_rows", "powerlaw", "banded_fem", "batch_uneven", "csr_to_coo_rows",
           "csr_to_csc", "compulsory_bytes"]
