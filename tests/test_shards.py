"""The reference's multi-GPU nnz split across processes (CPU only).

The library's partition, part row pointers and merge
(sblas_nnz_partition / sblas_part_rowptr / sblas_merge_parts, driven by
shards.dist_csrmv) against the oracle's restatement of spMV_mgpu_v1's split
and merge (src/dspmv_mgpu_v1.cu:120-152, :183-193, :304-319): cut points and
flags equal, merged y bit for bit, on the golden cases and on random
matrices with empty rows and rows spanning several parts.  The process-group
path runs world-size 2 and 3 groups over gloo on 127.0.0.1, each rank
computing its part with the oracle's row loop (the per-part product that a
GPU rank runs on its device), so the partition, exchange and merge logic is
covered without a GPU.
"""
import os
import socket

import numpy as np
import pytest

from conftest import golden_cases, load_golden


def _rand_csr(rng, m, n, mean, long_rows=(), empty_frac=0.2):
    deg = rng.poisson(mean, m)
    deg[rng.random(m) < empty_frac] = 0
    for r, d in long_rows:
        deg[r] = d
    rowptr = np.zeros(m + 1, np.int32)
    rowptr[1:] = np.cumsum(deg)
    nnz = int(rowptr[-1])
    col = np.concatenate([np.sort(rng.choice(n, size=min(int(d), n), replace=False))
                          for d in deg]).astype(np.int32) if nnz else np.zeros(0, np.int32)
    rowptr[1:] = np.cumsum(np.minimum(deg, n))
    val = rng.standard_normal(int(rowptr[-1]))
    return rowptr, col, val


def _cases():
    rng = np.random.default_rng(77)
    out = []
    for name in golden_cases():
        g = load_golden(name)
        if int(g["rowptr"][-1]) == 0:
            continue
        out.append((name, int(g["m"]), int(g["n"]), g["rowptr"], g["col"], g["val"], g["x"],
                    g["y0"], float(g["alpha"]), float(g["beta"])))
    for i, (m, n, mean, longs) in enumerate([(500, 300, 4.0, ()), (2000, 5000, 1.0, ()),
                                            (300, 4000, 3.0, ((7, 3000), (150, 2500))),
                                            (64, 64, 0.3, ())]):
        rp, c, v = _rand_csr(rng, m, n, mean, longs)
        x = rng.standard_normal(n)
        y0 = rng.standard_normal(m)
        out.append((f"rand{i}", m, n, rp, c, v, x, y0, 1.5, -0.75))
    return out


CASES = _cases()
NPARTS = (1, 2, 3, 4, 6, 8, 16)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_partition_and_merge_match_reference_split(sblas_lib, case):
    from hpda_sblas_pnnl_gb300 import shards
    from oracle import oracle as O
    name, m, n, rp, col, val, x, y0, alpha, beta = case
    nnz = int(rp[-1])
    for nparts in NPARTS:
        if nparts > nnz:
            continue
        parts = shards.partition(rp, nparts)
        ref = O.nnz_partition(m, rp, nparts)
        got = np.array([[p.start_idx, p.end_idx, p.start_row, p.end_row, p.start_flag,
                         p.end_flag, p.m] for p in parts], np.int32)
        np.testing.assert_array_equal(got, ref, err_msg=f"{name} nparts={nparts}")
        assert sum(p.nnz for p in parts) == nnz
        # every part computed with the oracle's row loop, then merged
        pieces = []
        for p in parts:
            prow = shards.part_rowptr(rp, p)
            assert prow[0] == 0 and prow[-1] == p.nnz and np.all(np.diff(prow) >= 0)
            lo, hi = p.start_idx, p.end_idx + 1
            pieces.append(O.csr_spmv(p.m, n, prow, np.ascontiguousarray(col[lo:hi]),
                                     np.ascontiguousarray(val[lo:hi]), x,
                                     y0[p.start_row: p.end_row + 1], alpha, beta))
        y = shards.merge(parts, pieces, beta, np.array(y0, dtype=np.float64))
        want = O.csr_spmv_nnz_split(m, n, rp, col, val, x, y0, nparts, alpha, beta)
        assert y.tobytes() == want.tobytes(), f"{name} nparts={nparts}"


def test_partition_rejects_bad_input(sblas_lib):
    from hpda_sblas_pnnl_gb300 import _lib, shards
    rp = np.array([0, 1, 3], np.int32)
    with pytest.raises(_lib.SblasError):
        shards.partition(rp, 4)            # 3 nonzeros cannot fill 4 parts
    with pytest.raises(_lib.SblasError):
        shards.partition(np.array([1, 2, 3], np.int32), 1)   # rowptr[0] != 0
    with pytest.raises(_lib.SblasError):
        shards.partition(rp, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, case_index, out_dir):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "tests"))
    import torch.distributed as dist

    from hpda_sblas_pnnl_gb300 import shards
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        name, m, n, rp, col, val, x, y0, alpha, beta = _cases()[case_index]

        def oracle_part(prow, pcol, pval, xx, py0, a, b):
            return O.csr_spmv(prow.size - 1, n, prow, np.ascontiguousarray(pcol),
                              np.ascontiguousarray(pval), xx, py0, a, b)

        y = np.array(y0, dtype=np.float64)
        shards.dist_csrmv(m, n, rp, col, val, x, y, alpha, beta, compute=oracle_part)
        np.save(os.path.join(out_dir, f"y{rank}.npy"), y)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_dist_csrmv_gloo_ranks_match_reference_split(sblas_lib, tmp_path, world):
    import torch.multiprocessing as mp

    from oracle import oracle as O
    idx = [c[0] for c in CASES].index("rand2")      # two long rows, empty rows
    name, m, n, rp, col, val, x, y0, alpha, beta = CASES[idx]
    mp.start_processes(_rank_main, args=(world, _free_port(), idx, str(tmp_path)),
                       nprocs=world, join=True, start_method="spawn")
    want = O.csr_spmv_nnz_split(m, n, rp, col, val, x, y0, world, alpha, beta)
    truth = O.csr_spmv(m, n, rp, col, val, x, y0, alpha, beta)
    parts = O.nnz_partition(m, rp, world)
    lo, hi = int(parts[0, 2]), int(parts[-1, 3]) + 1      # rows the parts hold
    assert hi < m                                          # the case has trailing empty rows
    for r in range(world):
        y = np.load(tmp_path / f"y{r}.npy")
        # the parts' rows: the reference's split and merge, bit for bit
        assert y[lo:hi].tobytes() == want[lo:hi].tobytes(), f"rank {r}"
        # outside them (empty rows the reference leaves untouched): beta*y0
        np.testing.assert_array_equal(y[:lo], beta * y0[:lo])
        np.testing.assert_array_equal(y[hi:], beta * y0[hi:])
        assert np.linalg.norm(y - truth) <= 1e-12 * np.linalg.norm(truth)


def _rank_main_gpu(rank, world, port, out_dir):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "tests"))
    import torch
    import torch.distributed as dist

    from hpda_sblas_pnnl_gb300 import shards
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("nccl", rank=rank, world_size=world)
    try:
        name, m, n, rp, col, val, x, y0, alpha, beta = _cases()[
            [c[0] for c in _cases()].index("rand2")]
        y = np.array(y0, dtype=np.float64)
        shards.dist_csrmv(m, n, rp, col, val, x, y, alpha, beta)   # the device product
        np.save(os.path.join(out_dir, f"y{rank}.npy"), y)
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_dist_csrmv_single_rank_nccl_on_device(sblas_lib, cuda, tmp_path):
    """One NCCL rank on the GPU: the part's product is the tile kernel."""
    import torch.multiprocessing as mp

    from oracle import oracle as O
    name, m, n, rp, col, val, x, y0, alpha, beta = CASES[[c[0] for c in CASES].index("rand2")]
    mp.start_processes(_rank_main_gpu, args=(1, _free_port(), str(tmp_path)), nprocs=1,
                       join=True, start_method="spawn")
    y = np.load(tmp_path / "y0.npy")
    truth = O.csr_spmv(m, n, rp, col, val, x, y0, alpha, beta)
    assert np.linalg.norm(y - truth) <= 1e-12 * np.linalg.norm(truth)
