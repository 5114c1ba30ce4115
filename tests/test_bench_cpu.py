"""The benchmark's host logic without a GPU: the reference arm's contract
line, its behaviour on ranks other than 0, the MatrixMarket reader timing
mode, and the max-over-ranks timing of the multi-rank path on a two-process
gloo group."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def run_bench(args, env_extra=None, timeout=600):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True,
                          text=True, cwd=ROOT, env=env, timeout=timeout)


def test_reference_arm_small_case_prints_the_contract_line():
    r = run_bench(["--impl", "reference", "--m", "20000", "--steps", "2", "--warmup", "3"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "GB/s" and d["value"] > 0
    assert d["steps"] == 2 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["m"] == 20000
    # inputs drawn where the GPU arm draws them when a GPU is present
    import torch
    assert d["config"]["generated_on"] == ("cuda" if torch.cuda.is_available() else "cpu")


def test_mmio_mode_times_both_readers_and_checks_parity():
    r = run_bench(["--mmio", "30000"])
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert d["mode"] == "mmio" and d["nnz"] == 30000 and d["bit_identical"] is True
    for leg in ("library_all_threads", "library_one_thread", "reference_fscanf_loop"):
        assert d[leg]["s"] > 0 and d[leg]["mb_s"] > 0


def test_reference_arm_other_ranks_exit_quietly():
    r = run_bench(["--impl", "reference", "--m", "20000"],
                  {"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, "cpu")
    q.put((rank, ms, bench.job_value(1_000_000_000, ms, world)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_on_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time; the job moves 2 x 1 GB per step
    assert [o[1] for o in out] == [15.0, 15.0]
    assert all(abs(o[2] - 2e9 / 15e-3 / 1e9) < 1e-9 for o in out)
