"""Writes the golden fixtures of tests/golden/ from the REFERENCE'S OWN CPU code.

The reference's csr_spmv_cpu (test/dspmv_test_smt.cu:39-52), coo_spmv_cpu
(test/dspmv_test_dgx1.cu:55-69), get_row_from_index, findFirstInSorted and
findLastInSorted (src/spmv_helper.cu) are compiled from its sources by
oracle/ref_build.sh into oracle/_ref/libref_cpu.so; this script runs them on
seeded inputs and stores inputs and outputs as small .npz files.  The COO ->
CSR/CSC conversions of the inputs use the oracle's stable counting sort
(the reference's conversion needs cuSPARSE).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def csr_from_rows(m, n, rows):
    """rows: list of (cols, vals) per row -> rowptr, col, val (int32/float64)."""
    rowptr = np.zeros(m + 1, np.int32)
    cols, vals = [], []
    for i, (c, v) in enumerate(rows):
        rowptr[i + 1] = rowptr[i] + len(c)
        cols.extend(c)
        vals.extend(v)
    return rowptr, np.asarray(cols, np.int32), np.asarray(vals, np.float64)


def coo_of(m, rowptr):
    return np.repeat(np.arange(m, dtype=np.int32), np.diff(rowptr)).astype(np.int32)


def save_case(name, m, n, rowptr, col, val, x, y0, alpha, beta):
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    y0 = np.ascontiguousarray(y0, np.float64)
    y_csr = O.ref_csr_spmv(m, n, rowptr, col, val, x, y0, alpha, beta)
    row = coo_of(m, rowptr)
    y_coo = O.ref_coo_spmv(m, n, row, col, val, x, y0, alpha, beta)
    cscval, colptr, cscrow = O.coo2csc(m, n, val, row, col)
    np.savez_compressed(OUT / f"{name}.npz", m=m, n=n, rowptr=rowptr, col=col, val=val, x=x,
                        y0=y0, alpha=alpha, beta=beta, y_ref_csr=y_csr, y_ref_coo=y_coo,
                        coo_row=row, csc_colptr=colptr, csc_row=cscrow, csc_val=cscval)
    print(f"{name}: m={m} n={n} nnz={col.size}")


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref/libref_cpu.so missing: run oracle/ref_build.sh first")
    rng = np.random.default_rng(20261203)

    # 1. the reference's 'g' matrix at n = 200 (test/dspmv_test_smt.cu:176-232),
    #    x = 1, alpha = 1, beta = 0, y0 = 0 as in the test programs (:356-373, :446-458)
    r, c, v = O.gen_g(200)
    val, rowptr, col = O.coo2csr(200, 200, v, r, c)
    save_case("g200", 200, 200, rowptr, col, val, np.ones(200), np.zeros(200), 1.0, 0.0)

    # 2. Zipf(1.5) rows at n = 200, U(-1, 1) values and x (config: g mode, n=200)
    n = 200
    k = np.arange(1, n + 1, dtype=np.float64)
    cdf = np.cumsum(k ** -1.5)
    cdf /= cdf[-1]
    deg = np.minimum(np.searchsorted(cdf, rng.random(n)), n - 1) + 1
    rows = []
    for i in range(n):
        cs = np.sort(rng.choice(n, size=int(deg[i]), replace=False))
        rows.append((cs, rng.uniform(-1, 1, cs.size)))
    rowptr, col, val = csr_from_rows(n, n, rows)
    x = rng.uniform(-1, 1, n)
    save_case("zipf200", n, n, rowptr, col, val, x, np.zeros(n), 1.0, 0.0)
    save_case("zipf200_ab", n, n, rowptr, col, val, x, rng.uniform(-1, 1, n), 1.5, -0.75)

    # 3. edge cases
    #  empty rows at the start, middle and end; rectangular
    m, n = 40, 33
    rows = []
    for i in range(m):
        if i < 3 or 17 <= i < 22 or i >= 36:
            rows.append(([], []))
        else:
            cs = np.sort(rng.choice(n, size=int(rng.integers(1, 9)), replace=False))
            rows.append((cs, rng.normal(size=cs.size)))
    rowptr, col, val = csr_from_rows(m, n, rows)
    save_case("empty_rows", m, n, rowptr, col, val, rng.normal(size=n), rng.normal(size=m),
              2.0, 0.5)
    #  one long row among short ones (a row spanning many thread chunks and tiles)
    m, n = 64, 8000
    rows = []
    for i in range(m):
        if i == 37:
            cs = np.arange(0, n, dtype=np.int64)
        else:
            cs = np.sort(rng.choice(n, size=int(rng.integers(0, 4)), replace=False))
        rows.append((cs, rng.uniform(-1, 1, cs.size)))
    rowptr, col, val = csr_from_rows(m, n, rows)
    save_case("long_row", m, n, rowptr, col, val, rng.uniform(-1, 1, n), np.zeros(m), 1.0, 0.0)
    #  1 x 1
    save_case("one", 1, 1, np.array([0, 1]), np.array([0]), np.array([3.5]), np.array([-2.0]),
              np.array([7.0]), 1.0, 1.0)
    #  no nonzeros: y = beta * y
    m = 17
    save_case("nnz0", m, 5, np.zeros(m + 1), np.zeros(0), np.zeros(0), rng.normal(size=5),
              rng.normal(size=m), 1.0, 0.25)
    #  one nonzero per row (tile kernels: many rows per tile)
    m = 3000
    rowptr = np.arange(m + 1)
    save_case("diag3000", m, m, rowptr, rng.permutation(m), rng.normal(size=m),
              rng.normal(size=m), np.zeros(m), 1.0, 0.0)
    #  a long run of empty rows inside one tile (more rows than a tile holds)
    m, n = 12000, 100
    rows = [([], []) for _ in range(m)]
    for i in list(range(0, 50)) + list(range(11950, 12000)):
        cs = np.sort(rng.choice(n, size=int(rng.integers(1, 30)), replace=False))
        rows[i] = (cs, rng.normal(size=cs.size))
    rowptr, col, val = csr_from_rows(m, n, rows)
    save_case("sparse_rows", m, n, rowptr, col, val, rng.normal(size=n), rng.normal(size=m),
              -1.0, 2.0)

    # 4. partition helpers on sorted arrays with repeats
    a = np.sort(rng.integers(0, 50, size=200)).astype(np.int32)
    a[0] = 0
    keys = np.arange(-2, 53, dtype=np.int32)
    first = np.array([O.ref_find_first_in_sorted(a, a.size - 1, int(k)) for k in keys], np.int32)
    last = np.array([O.ref_find_last_in_sorted(a, a.size - 1, int(k)) for k in keys], np.int32)
    rp = np.load(OUT / "empty_rows.npz")["rowptr"]
    idx = np.arange(0, int(rp[-1]), dtype=np.int32)
    rowof = np.array([O.ref_get_row_from_index(rp.size - 1, rp, int(i)) for i in idx], np.int32)
    np.savez_compressed(OUT / "search.npz", a=a, keys=keys, first=first, last=last, rowptr=rp,
                        idx=idx, row_of=rowof)
    print("search: done")


if __name__ == "__main__":
    main()
