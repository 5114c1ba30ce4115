"""Benchmark of the FP64 SpMV hot path on GB300 (one JSON line on stdout).

Workload (the power-law configuration): y = 1.0*A*x + 0.0*y, A a 4.0M x 4.0M
power-law graph with ~70M nonzeros (out-degree exponent 2.1, max row 20k),
values 1.0 FP64, x ~ U(0,1), int32 CSR indices.  One step = one SpMV over
the whole matrix through sblas_dcsrmv (tile partition + tile kernel + carry
fix-up; 3 launches), inputs resident in HBM.  The compulsory bytes (~920 MB:
val, col, rowptr, x read once, y written once) exceed the 129 MB L2, so no
flush is needed between steps; x (32 MB) stays L2-resident by design.

  value        compulsory GB/s of the whole job (all ranks) over the timed steps
  e2e          same metric through the reference-facing C ABI
               (spMV_mgpu_baseline) from pinned HOST buffers: host->device
               copies of the matrix and x, the SpMV, the device->host copy of
               y, all inside the timed region
  roofline     the tile kernel (with its carry fix-up) timed alone with CUDA
               events on its stream; peak = MEASURED_PEAKS.json hbm_gbs
  cpu_baseline the reference's CPU loop (oracle/_ref when built on this
               machine, else its restatement in oracle/) on all host cores

python bench.py --gpus N --steps K --warmup W [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SpMV HBM GB/s & % roofline: plain FP64 vs mixed/batched/fwd+bwd at stated err"
WORKLOAD = ("power-law graph 4.0M x 4.0M, ~70M nnz (exponent 2.1, max row 20k), values 1.0 "
            "FP64, x~U(0,1); FP64 CSR y=1.0*A*x+0.0*y")
FALLBACK_HBM = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-extras", action="store_true", help="skip the other forms")
    p.add_argument("--forms", default="banded,pattern,coo,batch,autograd",
                   help="comma list of the other forms to measure")
    p.add_argument("--seed", type=int, default=2021)
    p.add_argument("--m", type=int, default=4_000_000,
                   help="rows of the power-law matrix (smaller only for profiling captures)")
    p.add_argument("--sigma", type=int, default=0, help="tile shape (0 = library default)")
    p.add_argument("--kernel-only", action="store_true",
                   help="time the device steps only (no e2e, CPU baseline, extras): the "
                        "small case used for ncu captures")
    p.add_argument("--matrix", default="powerlaw", choices=["powerlaw", "banded"],
                   help="with --kernel-only: the matrix of the profiled case (banded: the "
                        "FEM-like generator, --m rows)")
    p.add_argument("--values", default="f64", choices=["f64", "f32"],
                   help="with --kernel-only: FP64 values or FP32 values (FP64 sums)")
    p.add_argument("--mmio", type=int, default=0, metavar="NNZ",
                   help="host only: time the MatrixMarket reader on a seeded coordinate file "
                        "of NNZ real entries against the reference's per-entry fscanf loop")
    p.add_argument("--mmio-digits", type=int, default=17, choices=range(1, 18), metavar="D",
                   help="with --mmio: significant digits of the written values (17: every "
                        "double round-trips; 16 or fewer: the reader's exact short path)")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(v: float, device) -> float:
    """The maximum of v over the ranks of the initialised process group (v
    itself without one): the job's time is its slowest rank's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(v)
    t = torch.tensor([float(v)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(bytes_per_rank: int, ms_step: float, world: int) -> float:
    """Whole-job compulsory GB/s: every rank moves bytes_per_rank per step
    (weak scaling, an independent instance per rank)."""
    return world * bytes_per_rank / (ms_step * 1e-3) / 1e9


def peaks():
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [s.strip() for s in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(device, seed, m=4_000_000):
    from hpda_sblas_pnnl_gb300 import synth
    a, x = synth.powerlaw(m=m, seed=seed, device=device)
    return a, x


def cpu_time_spmv(a_np, x_np, m, n, reps, threads, use_ref, warmup=2):
    """Median seconds of the reference CPU loop on `threads` host threads."""
    import numpy as np
    from oracle import oracle as O
    rp, col, val = a_np
    y0 = np.zeros(m)
    fn = (lambda: O.ref_csr_spmv(m, n, rp, col, val, x_np, y0, 1.0, 0.0, threads=threads)) \
        if use_ref else \
        (lambda: O.csr_spmv(m, n, rp, col, val, x_np, y0, 1.0, 0.0, threads=threads))
    for _ in range(warmup):
        fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts), ts


def run_reference(args):
    """--impl reference: the reference's own CPU SpMV (csr_spmv_cpu,
    test/dspmv_test_smt.cu:39-52) on all host cores, same workload/metric."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    import torch
    from hpda_sblas_pnnl_gb300 import synth
    from oracle import oracle as O
    O.build() if not O.LIB.exists() else None
    # The same seeded matrix as the GPU arm: generated with the same device's
    # random streams (torch's CPU and CUDA generators differ), then copied to
    # host memory.  Only input generation touches the GPU; the timed loop is
    # the reference's CPU code.
    gen_dev = "cuda" if torch.cuda.is_available() else "cpu"
    try:
        a, x = make_workload(gen_dev, args.seed, args.m)
        a, x = a.to("cpu"), x.cpu()
    except (RuntimeError, torch.cuda.OutOfMemoryError):
        gen_dev = "cpu"   # inputs only: same distribution, another random stream
        a, x = make_workload(gen_dev, args.seed, args.m)
    if torch.cuda.is_available():
        torch.cuda.empty_cache()
    m, n, nnz = a.m, a.n, a.nnz
    a_np = tuple(np.ascontiguousarray(t) for t in a.numpy())
    x_np = np.ascontiguousarray(x.numpy())
    threads = os.cpu_count() or 1
    use_ref = O.ref_available()
    bytes_step = synth.compulsory_bytes(m, n, nnz)
    warm = max(args.warmup, 3)
    med, ts = cpu_time_spmv(a_np, x_np, m, n, max(args.steps, 1), threads, use_ref, warm)
    # warmup and steps: every step is one full SpMV (a bounded sample: the
    # whole matrix, ~0.01-1 s per step on the host)
    total = sum(ts)
    value = bytes_step * len(ts) / total / 1e9
    kind = "reference" if use_ref else "port"
    sample = f"full matrix ({nnz} nnz), {len(ts)} steps after {warm} warm-up runs"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s",
        "n_gpus": ws, "steps": len(ts), "warmup": warm, "ms_per_step": round(1e3 * total / len(ts), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded power-law stand-in for the reference's SuiteSparse graphs)",
        "config": {"workload": WORKLOAD, "m": m, "n": n, "nnz": nnz,
                   "bytes_per_step": bytes_step, "host_threads": threads,
                   "generated_on": gen_dev},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads,
                         "kind": kind, "sample": sample,
                         "gflops": round(2 * nnz * len(ts) / total / 1e9, 3)},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cuda_event_ms(fn, stream, reps):
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(reps)]
    for e0, e1 in ev:
        e0.record(stream)
        fn()
        e1.record(stream)
    torch.cuda.synchronize()
    return [e0.elapsed_time(e1) for e0, e1 in ev]


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist
    from hpda_sblas_pnnl_gb300 import _lib, api, ops, synth

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load(build_if_missing=True)
    stream = torch.cuda.current_stream(dev)

    # each rank holds its own full-size instance (weak scaling, no collective
    # on the data path): rank r uses seed + r
    if args.kernel_only and args.matrix == "banded":
        a, x = synth.banded_fem(m=args.m, seed=args.seed + rank, device=dev)
    else:
        a, x = make_workload(dev, args.seed + rank, args.m)
    if args.kernel_only and args.values == "f32":
        a.val = a.val.float()
    m, n, nnz = a.m, a.n, a.nnz
    y = torch.zeros(m, dtype=torch.float64, device=dev)
    bytes_step = synth.compulsory_bytes(m, n, nnz, val_bytes=a.val.element_size())
    kernel = ops.KERNEL_MERGEPATH
    # tile shape: --sigma, else the library default for --kernel-only (the
    # profiling case), else the autotuner's measured pick on this matrix
    sigma_times = None
    if args.sigma > 0:
        sigma = args.sigma
    elif args.kernel_only:
        sigma = ops.default_sigma(m, nnz)
    else:
        from hpda_sblas_pnnl_gb300 import tune
        sigma, sigma_times = tune.tile_sigma(a.rowptr, a.col, a.val, x)
    work = torch.empty(ops.workspace_bytes(nnz, sigma), dtype=torch.uint8, device=dev)

    def step():
        ops.csrmv(a.rowptr, a.col, a.val, x, y, 1.0, 0.0, kernel=kernel, sigma=sigma, work=work)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)  # let the sampler start before the timed region
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), dev)
    ms_step = ms / args.steps
    value = job_value(bytes_step, ms_step, ws)
    launches_per_step = 3

    # correctness of what was timed (oracle spot check on rank 0 is in the
    # tests; here a cheap invariant: sum(y) = sum over nonzeros of val * x[col])
    tot = float((a.val.double() * x[a.col.to(torch.int64)]).sum())
    chk = abs(float(y.sum()) - tot) / max(abs(tot), 1e-300)

    out = {}
    if rank == 0 and args.kernel_only:
        print(json.dumps({"metric": METRIC, "value": round(value, 2), "unit": "GB/s",
                          "n_gpus": ws, "steps": args.steps, "ms_per_step": round(ms_step, 4),
                          "config": {"matrix": args.matrix, "values": args.values, "m": m,
                                     "nnz": nnz, "sigma": sigma, "bytes_per_step": bytes_step,
                                     "check_rel_err": chk},
                          "note": "kernel-only small case (profiling); not the benchmark line"}),
              flush=True)
    elif rank == 0:
        # ---- roofline: tile kernel (+ carry fix-up) alone, analysed plan
        plan = ops.CsrPlan(a.rowptr, a.col, a.val, kernel=kernel, sigma=sigma)
        for _ in range(3):
            plan(x, y)
        kt = cuda_event_ms(lambda: plan(x, y), stream, 20)
        k_ms = statistics.mean(kt)
        pk, pk_kind = peaks()
        achieved = bytes_step / (k_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": pk, "unit": "GB/s",
                "frac": round(achieved / pk, 4), "traffic": None, "peak_source": pk_kind,
                "kernel": f"tile_spmv_kernel<128,{sigma},F64> + tile_fixup_kernel",
                "kernel_us": round(k_ms * 1e3, 2),
                "kernel_gflops": round(2 * nnz / (k_ms * 1e-3) / 1e9, 2),
                "bounds_note": "1 DFMA per nonzero at the measured 5.3e11 DFMA/s caps this matrix "
                               f"at {5.3e11 * bytes_step / nnz / 1e9:.0f} GB/s; one random L2 "
                               "gather per nonzero at the measured 2.8e11/s caps it at "
                               f"{2.8e11 * bytes_step / nnz / 1e9:.0f} GB/s"}
        traffic_file = ROOT / "profiles" / "traffic.json"
        if traffic_file.exists():
            try:
                tr = json.loads(traffic_file.read_text())
                roof["traffic"] = tr.get("powerlaw_fp64_bytes_per_launch")
            except Exception:
                pass

        # ---- e2e through the reference-facing C ABI with pinned host buffers
        rp_h = a.rowptr.cpu().pin_memory().numpy()
        col_h = a.col.cpu().pin_memory().numpy()
        val_h = a.val.cpu().pin_memory().numpy()
        x_h = x.cpu().pin_memory().numpy()
        y_h = torch.zeros(m, dtype=torch.float64).pin_memory().numpy()
        for _ in range(2):
            api.spMV_mgpu_baseline(m, n, nnz, 1.0, val_h, rp_h, col_h, x_h, 0.0, y_h)
        e2e_steps = max(3, min(args.steps, 10))
        t0 = time.perf_counter()
        rets = []
        for _ in range(e2e_steps):
            rets.append(api.spMV_mgpu_baseline(m, n, nnz, 1.0, val_h, rp_h, col_h, x_h, 0.0, y_h))
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        h2d = 8 * nnz + 4 * nnz + 4 * (m + 1) + 8 * n
        d2h = 8 * m
        e2e = {"value": round(bytes_step / e2e_s / 1e9, 3), "unit": "GB/s",
               "gflops": round(2 * nnz / e2e_s / 1e9, 3),
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": round(e2e_s * 1e3, 3),
               "comm_ms": round(1e3 * statistics.mean(r.comm_time for r in rets), 3),
               "comp_ms": round(1e3 * statistics.mean(r.comp_time for r in rets), 3),
               "api": "spMV_mgpu_baseline (include/spmv_kernel.h)"}
        e2e_err = float(np.abs(y_h - y.cpu().numpy()).max())

        # ---- CPU baseline (bounded sample: a few full SpMVs, all host cores)
        cpu = None
        if ws == 1:
            from oracle import oracle as O
            if not O.LIB.exists():
                O.build()
            threads = os.cpu_count() or 1
            use_ref = O.ref_available()
            a_np = (rp_h, col_h, val_h)
            med, ts = cpu_time_spmv(a_np, x_h, m, n, 8, threads, use_ref)
            cpu = {"value": round(bytes_step / med / 1e9, 3), "unit": "GB/s", "cores": threads,
                   "gflops": round(2 * nnz / med / 1e9, 3),
                   "kind": "reference" if use_ref else "port",
                   "sample": f"8 full SpMVs of the same matrix (median), {threads} threads"}

        extras = {}
        if not args.no_extras:
            extras = run_extras(dev, stream, args)
            if "powerlaw_csc" in extras:   # per-call CSC against the CSR step above
                extras["powerlaw_csc"]["time_vs_csr_step"] = round(
                    extras["powerlaw_csc"]["us"] / (ms_step * 1e3), 3)

        out = {
            "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": ws,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(ms_step, 4),
            "gflops": round(2 * nnz * ws / (ms_step * 1e-3) / 1e9, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded power-law stand-in for the reference's SuiteSparse graphs)",
            "config": {"workload": WORKLOAD, "m": m, "n": n, "nnz": nnz,
                       "bytes_per_step": bytes_step, "kernel": "2 (nnz tiles)", "sigma": sigma,
                       "sigma_tuner_ms": ({str(k): round(v, 4) for k, v in sigma_times.items()}
                                          if sigma_times else None),
                       "l2": f"inputs larger than L2 ({bytes_step / 1e6:.0f} MB > 129 MB), no flush",
                       "launches": "tile partition + tile kernel + carry fix-up",
                       "check_rel_err": chk, "e2e_max_abs_diff": e2e_err},
            "roofline": roof, "e2e": e2e, "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": launches_per_step * args.steps,
        }
        if extras:
            out["forms"] = extras
        print(json.dumps(out), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def run_extras(dev, stream, args):
    """The other forms, each timed with CUDA events (analysed plans): banded
    FP64 and FP32 values, pattern-only and COO power-law (errors: relative
    L2 against the FP64 oracle on the same inputs), the batched uneven SpMM
    and the differentiable SpMM (see their functions)."""
    import numpy as np
    import torch
    from hpda_sblas_pnnl_gb300 import ops, synth
    from oracle import oracle as O
    pk, _ = peaks()
    res = {}
    threads = os.cpu_count() or 1

    def timed(plan, x, y, reps=10):
        for _ in range(3):
            plan(x, y)
        return statistics.mean(cuda_event_ms(lambda: plan(x, y), stream, reps))

    forms = set(args.forms.split(","))
    if "banded" in forms:
        res.update(run_banded_extra(dev, stream, args, timed, threads, pk))
    if "pattern" in forms or "coo" in forms:
        res.update(run_powerlaw_forms_extra(dev, stream, args, timed, threads, pk, forms))
    if "batch" in forms:
        res["batched"] = run_batch_extra(dev, stream, args)
        torch.cuda.empty_cache()
    if "autograd" in forms:
        res["autograd"] = run_autograd_extra(dev, stream, args)
        torch.cuda.empty_cache()
    return res


def run_banded_extra(dev, stream, args, timed, threads, pk):
    import numpy as np
    import torch
    from hpda_sblas_pnnl_gb300 import ops, synth, tune
    from oracle import oracle as O
    res = {}
    a, x = synth.banded_fem(device=dev)
    m, n, nnz = a.m, a.n, a.nnz
    rp, c, v = a.numpy()
    ref = O.csr_spmv(m, n, rp, c, v, x.cpu().numpy(), np.zeros(m), threads=threads)
    nref = np.linalg.norm(ref)
    y = torch.zeros(m, dtype=torch.float64, device=dev)
    for name, val, vb in (("banded_fp64", a.val, 8), ("banded_fp32val", a.val.float(), 4)):
        sg, _ = tune.tile_sigma(a.rowptr, a.col, val, x)
        plan = ops.CsrPlan(a.rowptr, a.col, val, sigma=sg)
        ms = timed(plan, x, y)
        err = float(np.linalg.norm(y.cpu().numpy() - ref) / nref)
        b = synth.compulsory_bytes(m, n, nnz, val_bytes=vb)
        res[name] = {"gbs": round(b / ms / 1e6, 1), "frac": round(b / ms / 1e6 / pk, 4),
                     "gflops": round(2 * nnz / ms / 1e6, 1),
                     "us": round(ms * 1e3, 1), "bytes": b, "rel_l2_err": err, "nnz": nnz,
                     "sigma": sg}
        del plan
    if "banded_fp64" in res and "banded_fp32val" in res:
        res["fp32val_speedup"] = round(res["banded_fp64"]["us"] / res["banded_fp32val"]["us"], 3)
    del a, x, y
    torch.cuda.empty_cache()
    return res


def run_powerlaw_forms_extra(dev, stream, args, timed, threads, pk, forms):
    import numpy as np
    import torch
    from hpda_sblas_pnnl_gb300 import ops, synth, tune
    from oracle import oracle as O
    res = {}
    a, x = synth.powerlaw(m=args.m, seed=args.seed, device=dev)
    y = torch.zeros(a.m, dtype=torch.float64, device=dev)
    sg, _ = tune.tile_sigma(a.rowptr, a.col, None, x)
    plan = ops.CsrPlan(a.rowptr, a.col, None, sigma=sg)
    ms = timed(plan, x, y)
    b = synth.compulsory_bytes(a.m, a.n, a.nnz, val_bytes=0)
    rp, c, v = a.numpy()
    ref = O.csr_spmv(a.m, a.n, rp, c, v, x.cpu().numpy(), np.zeros(a.m), threads=threads)
    err = float(np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref))
    res["powerlaw_pattern"] = {"gbs": round(b / ms / 1e6, 1), "frac": round(b / ms / 1e6 / pk, 4),
                               "gflops": round(2 * a.nnz / ms / 1e6, 1),
                               "us": round(ms * 1e3, 1), "bytes": b, "rel_l2_err": err,
                               "sigma": sg}
    # CSC: the inspector (row-ordered structure by the library's bucket sort,
    # staging indices) timed apart from the executor (values moved into row
    # order + tile kernel); the one-shot call (both) beside them
    colptr, rowidx, cval = synth.csr_to_csc(a)
    for _ in range(2):
        plan_c = ops.CscPlan(a.m, colptr, rowidx)
    insp_ms = statistics.mean(cuda_event_ms(
        lambda: ops.CscPlan(a.m, colptr, rowidx), stream, 3))
    for _ in range(3):
        plan_c(cval, x, y)
    csc_ms = statistics.mean(cuda_event_ms(lambda: plan_c(cval, x, y), stream, 10))
    csc_err = float(np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref))
    plan_c.bind(cval)
    for _ in range(3):
        plan_c(None, x, y)
    bound_ms = statistics.mean(cuda_event_ms(lambda: plan_c(None, x, y), stream, 10))
    cw = plan_c.work
    for _ in range(2):
        ops.cscmv(colptr, rowidx, cval, x, y, work=cw)
    once_ms = statistics.mean(cuda_event_ms(
        lambda: ops.cscmv(colptr, rowidx, cval, x, y, work=cw), stream, 3))
    del plan_c, cw
    bcsc = synth.compulsory_bytes(a.m, a.n, a.nnz, fmt="csc")
    res["powerlaw_csc"] = {"gbs": round(bcsc / csc_ms / 1e6, 1),
                           "gflops": round(2 * a.nnz / csc_ms / 1e6, 1),
                           "frac": round(bcsc / csc_ms / 1e6 / pk, 4), "us": round(csc_ms * 1e3, 1),
                           "rel_l2_err": csc_err, "inspector_us": round(insp_ms * 1e3, 1),
                           "bound_values_us": round(bound_ms * 1e3, 1),
                           "one_shot_us": round(once_ms * 1e3, 1),
                           "note": "us/gbs: executor per call (values moved into row order "
                                   "through 8 MB staging buckets + tile kernel); inspector_us: "
                                   "row-ordered structure by the library's bucket sort and the "
                                   "staging indices, once per pattern; bound_values_us: "
                                   "executor with values kept in row order (sblas_csc_bind_values); "
                                   "one_shot_us: sblas_dcscmv (inspector without staging, "
                                   "values gathered directly, tile kernel)"}
    del colptr, rowidx, cval
    torch.cuda.empty_cache()
    row = synth.csr_to_coo_rows(a)
    rpw = torch.empty(a.m + 1, dtype=torch.int32, device=dev)
    coo_ms = statistics.mean(cuda_event_ms(
        lambda: ops.coomv(row, a.col, a.val, x, y, rowptr_work=rpw), stream, 10))
    bcoo = synth.compulsory_bytes(a.m, a.n, a.nnz, fmt="coo")
    res["powerlaw_coo"] = {"gbs": round(bcoo / coo_ms / 1e6, 1),
                           "gflops": round(2 * a.nnz / coo_ms / 1e6, 1),
                           "frac": round(bcoo / coo_ms / 1e6 / pk, 4), "us": round(coo_ms * 1e3, 1),
                           "note": "row pointer built on device each call, then tile kernel"}
    del a, x, y
    torch.cuda.empty_cache()
    return res


def run_batch_extra(dev, stream, args):
    """Batched uneven SpMM: 64 matrices (rows log-uniform in [10k, 1M], mean
    nonzeros per row log-uniform in [4, 64], half power-law, half banded),
    k in {1, 4, 8} right-hand sides ~ U(-1, 1).  One graph-captured run of
    the batched plan (s picked by the autotuner) against 64 * k launches of
    the single-matrix tile kernel (one per matrix and right-hand side,
    analysed plans, eager), and for k >= 2 against 64 launches of the k-column
    SpMM (one per matrix, ops.SpmmPlan), all timed with CUDA events; agreement
    of the results (relative L2) is the correctness check at this size."""
    import numpy as np
    import torch
    from hpda_sblas_pnnl_gb300 import ops, synth, tune
    pk, _ = peaks()
    mats = synth.batch_uneven(nmat=64, seed=args.seed + 64, device=dev)
    total_nnz = sum(a.nnz for a in mats)
    res = {"matrices": len(mats), "nnz": total_nnz,
           "rows": [min(a.m for a in mats), max(a.m for a in mats)]}
    single = [ops.CsrPlan(a.rowptr, a.col, a.val) for a in mats]
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed + 7)
    for k in (1, 4, 8):
        xs = [(torch.rand((a.n, k), generator=g, dtype=torch.float64, device=dev) * 2 - 1)
              for a in mats]
        if k == 1:
            xs = [x.view(-1) for x in xs]
        ys = [torch.zeros((a.m, k) if k > 1 else (a.m,), dtype=torch.float64, device=dev)
              for a in mats]
        trip = [(a.rowptr, a.col, a.val) for a in mats]
        s_best, s_times = tune.batch_s(trip, xs, k)
        plan = ops.BatchPlan(trip, xs, ys, k, s=s_best)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            plan()
        torch.cuda.current_stream(dev).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            plan()
        for _ in range(3):
            graph.replay()
        b_ms = statistics.median(cuda_event_ms(graph.replay, stream, 10))
        # per-matrix, per-column launches of the single-matrix kernel
        xc = [[x.view(x.shape[0], -1)[:, c].contiguous() for c in range(k)] for x in xs]
        yc = [[torch.zeros(a.m, dtype=torch.float64, device=dev) for _ in range(k)] for a in mats]

        def per_matrix():
            for p, xcs, ycs in zip(single, xc, yc):
                for c in range(k):
                    p(xcs[c], ycs[c])

        per_matrix()
        p_ms = statistics.median(cuda_event_ms(per_matrix, stream, 5))
        # the fair per-matrix arm for k >= 2: one k-column SpMM launch per
        # matrix (ops.SpmmPlan: same kernel family, one gather of X per nonzero)
        pm_spmm_ms = None
        if k > 1:
            splans = [ops.SpmmPlan(a.rowptr, a.col, a.val, n=a.n, k=k, s=s_best) for a in mats]
            ysp = [torch.zeros((a.m, k), dtype=torch.float64, device=dev) for a in mats]

            def per_matrix_spmm():
                for sp, xx, yy in zip(splans, xs, ysp):
                    sp(xx, yy)

            per_matrix_spmm()
            pm_spmm_ms = statistics.median(cuda_event_ms(per_matrix_spmm, stream, 5))
            for sp in splans:
                sp.close()
            del splans, ysp
        num = den = 0.0
        for y, ycs in zip(ys, yc):
            yy = y.view(y.shape[0], -1)
            for c in range(k):
                num += float(((yy[:, c] - ycs[c]) ** 2).sum())
                den += float((ycs[c] ** 2).sum())
        bytes_k = sum(synth.compulsory_bytes(a.m, a.n, a.nnz, k=k) for a in mats)
        flops = 2.0 * total_nnz * k
        res[f"k{k}"] = {
            "batched_ms": round(b_ms, 3), "per_matrix_ms": round(p_ms, 3),
            "speedup_vs_per_matrix": round(p_ms / b_ms, 3),
            "per_matrix_spmm_ms": None if pm_spmm_ms is None else round(pm_spmm_ms, 3),
            "speedup_vs_per_matrix_spmm": (None if pm_spmm_ms is None
                                           else round(pm_spmm_ms / b_ms, 3)),
            "gbs": round(bytes_k / b_ms / 1e6, 1), "frac_hbm": round(bytes_k / b_ms / 1e6 / pk, 4),
            "fp64_tflops": round(flops / b_ms / 1e9, 4), "s": s_best,
            "tuner_ms": {str(sv): round(t, 3) for sv, t in s_times.items()},
            "units": plan.units,
            "launches": ("1 graph (tile kernel over all 64 matrices + carry fix-up)" if k == 1
                         else "1 graph (batched kernel + carry fix-up)"),
            "per_matrix_launches": 64 * k * 2, "rel_l2_vs_per_matrix": (num / den) ** 0.5,
        }
        plan.close()
        del graph, xs, ys, xc, yc
        torch.cuda.empty_cache()
    return res


def run_autograd_extra(dev, stream, args):
    """Differentiable SpMM: 1.0M-row power-law CSR, ~20M nonzeros, values
    N(0, 1), X (n x 16) and upstream G (m x 16) N(0, 1).  forward = Y = A X;
    forward + backward = the same through autograd.spmm plus backward(G)
    (dX = A^T G and dval), measured with CUDA events, FP64 and FP32 values."""
    import torch
    from hpda_sblas_pnnl_gb300 import autograd, synth
    a, _ = synth.powerlaw(m=1_000_000, mean_deg=22.4, seed=args.seed + 5, device=dev,
                          values="normal")
    k = 16
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed + 9)
    x0 = torch.randn((a.n, k), generator=g, dtype=torch.float64, device=dev)
    gy = torch.randn((a.m, k), generator=g, dtype=torch.float64, device=dev)
    res = {"m": a.m, "nnz": a.nnz, "k": k}
    for name, dtype in (("fp64", torch.float64), ("fp32val", torch.float32)):
        op = autograd.CsrOperator(a.rowptr, a.col, a.n, k, value_dtype=dtype, s=None)
        val = a.val.to(dtype).requires_grad_(True)
        x = x0.clone().requires_grad_(True)
        y = torch.empty((a.m, k), dtype=torch.float64, device=dev)

        def fwd():
            op.fwd(x.detach(), y, val=val.detach())

        def fwd_bwd():
            val.grad = None
            x.grad = None
            autograd.spmm(op, val, x).backward(gy)

        for _ in range(3):
            fwd()
            fwd_bwd()
        f_ms = statistics.median(cuda_event_ms(fwd, stream, 10))
        fb_ms = statistics.median(cuda_event_ms(fwd_bwd, stream, 10))
        # the backward's parts alone: dX = A^T G (with the value permutation), dval
        dx_ms = statistics.median(cuda_event_ms(lambda: op.grad_x(val.detach(), gy), stream, 10))
        dv_ms = statistics.median(cuda_event_ms(lambda: op.grad_val(gy, x.detach()), stream, 10))
        vb = 8 if dtype == torch.float64 else 4
        fbytes = synth.compulsory_bytes(a.m, a.n, a.nnz, val_bytes=vb, k=k)
        res[name] = {"fwd_ms": round(f_ms, 3), "fwd_bwd_ms": round(fb_ms, 3),
                     "ratio": round(fb_ms / f_ms, 3),
                     "fwd_fp64_tflops": round(2.0 * a.nnz * k / f_ms / 1e9, 4),
                     "fwd_gbs": round(fbytes / f_ms / 1e6, 1),
                     "s_fwd": op.fwd.s, "s_bwd": op.bwd.s, "dx_ms": round(dx_ms, 3),
                     "dval_ms": round(dv_ms, 3)}
        del op, val, x, y
        torch.cuda.empty_cache()
    return res


def run_mmio(args):
    """--mmio NNZ: the library's MatrixMarket reader (sblas_mm_read_coo, all
    host threads and one) against the reference's reading loop (one fscanf
    per entry, test/dspmv_test_dgx1.cu:160-181, restated in the oracle) on a
    seeded real coordinate file: 1M x 1M, uniform indices, N(0, 1) values
    written with --mmio-digits significant digits (default 17).  The file is
    read from the page cache (written just before); results must agree bit
    for bit."""
    import tempfile

    import numpy as np
    from hpda_sblas_pnnl_gb300 import mmio
    from oracle import oracle as O
    O.build() if not O.LIB.exists() else None
    nz, m = int(args.mmio), 1_000_000
    vfmt = "%d %d %." + str(int(args.mmio_digits)) + "g\n"
    rng = np.random.default_rng(args.seed)
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "uniform_1m.mtx"
        with open(path, "w") as f:
            f.write("%%MatrixMarket matrix coordinate real general\n% seeded\n")
            f.write(f"{m} {m} {nz}\n")
            for s0 in range(0, nz, 1 << 20):
                k = min(nz, s0 + (1 << 20)) - s0
                r = rng.integers(1, m + 1, k)
                c = rng.integers(1, m + 1, k)
                v = rng.standard_normal(k)
                f.write("".join(vfmt % t for t in zip(r.tolist(), c.tolist(), v.tolist())))
        size = path.stat().st_size

        def timed(fn, reps):
            ts, out = [], None
            for _ in range(reps):
                t0 = time.perf_counter()
                out = fn()
                ts.append(time.perf_counter() - t0)
            return statistics.median(ts), out

        threads = os.cpu_count() or 1
        t_all, lib_all = timed(lambda: mmio.read_coo(path, threads=0), 3)
        t_one, lib_one = timed(lambda: mmio.read_coo(path, threads=1), 2)
        t_ref, ref = timed(lambda: O.mm_read_fscanf(path), 1)
    same = all(a.tobytes() == b.tobytes() and a.tobytes() == c.tobytes()
               for a, b, c in zip(lib_all[2:], lib_one[2:], ref[2:]))

    def leg(t, nthreads):
        return {"s": round(t, 4), "mb_s": round(size / t / 1e6, 1),
                "m_entries_s": round(nz / t / 1e6, 2), "threads": nthreads}

    print(json.dumps({
        "mode": "mmio", "file_bytes": size, "nnz": nz, "value_digits": int(args.mmio_digits),
        "library_all_threads": leg(t_all, threads), "library_one_thread": leg(t_one, 1),
        "reference_fscanf_loop": leg(t_ref, 1),
        "speedup_vs_reference": round(t_ref / t_all, 2), "bit_identical": bool(same)}),
        flush=True)
    if not same:
        sys.exit(1)


def main():
    args = parse()
    if args.mmio:
        run_mmio(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
