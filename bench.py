"""Benchmark of the sync-free sparse triangular solve on GB300.

Default workload (N=1): the plain FP64 solve of the 4,194,304-row wide-level
matrix (1-7 off-diagonals per row in a band of 65,536; b = L*ones), the
configuration the headline metric is quoted on.  One step = one complete
solve (fill of x + the solve kernel) over inputs already resident in HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]
                  [--workload wide_4m|plain_20k|zipf_1m|grad_1m|batched|autograd]
                  [--dtype f64|f32]

Output: one JSON line on rank 0.  `value` is GFLOP/s with (2*nnz - n) flops
per solve (the benchmark definition's convention); `roofline` relates the
solve kernel's algorithmic bytes (4(n+1) + 4nnz + 4n + s*nnz + 2*s*n, the
reference's formula in CUDA/ourWrtFst/spts_syncfree_cuda_csr_wrt.h:208) per
launch to its CUDA-event duration; `e2e` is the same metric through the
host-buffer C-ABI call (capsp_solve_host: H2D of b, solve, D2H of x);
`cpu_baseline` is the reference's serial executor on the host cores.
--impl reference times the reference's own CPU implementation instead.
Multi-GPU: the solve is one dependency DAG and does not shard; --gpus N runs
N independent replicas (one process per GPU) and reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="wide_4m")
    ap.add_argument("--dtype", default="f64", choices=["f64", "f32"])
    ap.add_argument("--nrhs", type=int, default=0, help="right-hand sides (batched/autograd workloads)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def algorithmic_bytes(n: int, nnz: int, s: int, k: int = 1) -> float:
    """rowptr + colidx + flags + values + b and x (reference formula, k RHS)."""
    return 4.0 * (n + 1) + 4.0 * nnz + 4.0 * n + s * nnz + 2.0 * s * n * k


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(kernel: str, workload: str):
    """dram bytes per launch from a committed ncu summary (profiles/<kernel>_<workload>.txt)."""
    p = ROOT / "profiles" / f"{kernel}_{workload}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            return float(line.split(":", 1)[1].split()[0])
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def workload_matrix(name: str, dtype):
    import capellinisptrsv_gb300 as cs
    m = cs.generate(name, seed=0)
    val = m.val.astype(dtype)
    _, b = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, val)
    return m, val, b


def cpu_arm_runner(m, val):
    """The reference's serial executor (oracle/_ref when built here, else the oracle port)."""
    import oracle
    ref = oracle.ref()
    if ref is not None:
        return ref.prepared_forward(m.rowptr, m.colidx, val), "reference"
    return oracle.prepared_forward(m.rowptr, m.colidx, val), "port"


def time_cpu(run, b, seconds: float, min_reps: int = 3):
    x = np.empty_like(b)
    times = []
    t_end = time.perf_counter() + seconds
    while len(times) < min_reps or time.perf_counter() < t_end:
        t0 = time.perf_counter()
        run(b, x)
        times.append(time.perf_counter() - t0)
    return times, x


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU implementation of the path
# ---------------------------------------------------------------------------

def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    dt = np.float64 if args.dtype == "f64" else np.float32
    m, val, b = workload_matrix(args.workload, dt)
    run, kind = cpu_arm_runner(m, val)
    x = np.empty_like(b)
    for _ in range(args.warmup):
        run(b, x)
    steps = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        run(b, x)
        steps.append(time.perf_counter() - t0)
    flops = 2.0 * m.nnz - m.n
    sec = sum(steps) / len(steps)
    val_gf = flops / sec / 1e9
    line = {
        "impl": "reference", "metric": "SpTRSV GFLOP/s (2*nnz-n flops per solve)", "value": val_gf,
        "unit": "GFLOP/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": args.dtype, "data": "synthetic (seeded generator, seed 0)",
        "config": {"workload": args.workload, "n": m.n, "nnz": m.nnz, "rhs": 1,
                   "l2": "host run; inputs larger than the last-level cache"},
        "cpu_baseline": {"value": val_gf, "unit": "GFLOP/s", "cores": 1, "kind": kind,
                         "sample": f"{args.steps} full serial solves of the {args.workload} matrix "
                                   "(sptrsv_syncfree_executor FORWARD; transpose and in-degree analysis excluded)"},
        "e2e": {"value": val_gf, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gflops_2nnz": 2.0 * m.nnz / sec / 1e9, "host_cores_available": os.cpu_count(),
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# native arm
# ---------------------------------------------------------------------------

def run_native(args):
    import torch
    import capellinisptrsv_gb300 as cs
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    dt = np.float64 if args.dtype == "f64" else np.float32
    s_bytes = 8 if dt == np.float64 else 4
    m, val, b = workload_matrix(args.workload, dt)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    rp_d, ci_d, val_d, b_d = to(m.rowptr), to(m.colidx), to(val), to(b)
    solver = cs.TriangularSolver(rp_d, ci_d, val_d)
    solver.set_profiling(True)
    x_d = torch.empty_like(b_d)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    for _ in range(args.warmup):
        solver.solve(b_d, x_d)
    solver.status()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kern_ms = []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index if dev.index is not None else 0) as clk:
        t_wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()                      # L2 flush outside the timed events
            ev[i][0].record(stream)
            solver.solve(b_d, x_d)
            ev[i][1].record(stream)
            kern_ms.append(solver.last_kernel_ms())
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    if world > 1:
        torch.distributed.barrier()
    solver.status()
    step_ms = [a.elapsed_time(bb) for a, bb in ev]
    ms = sum(step_ms) / len(step_ms)
    kms = sum(kern_ms) / len(kern_ms)
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([ms, kms], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms, kms = float(tt[0]), float(tt[1])

    # correctness spot-check against the reference's self-check (x_ref = ones)
    xh = x_d.cpu().numpy()
    max_dev = float(np.max(np.abs(xh - 1.0)))

    flops = 2.0 * m.nnz - m.n
    value = world * flops / (ms * 1e-3) / 1e9
    alg_bytes = algorithmic_bytes(m.n, m.nnz, s_bytes)
    peak, peak_kind = peaks()
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    traffic = profile_traffic("row_solve", args.workload + "_" + args.dtype)

    line = None
    if rank == 0:
        e2e = None
        if not args.no_e2e:
            e2e = e2e_measure(cs, m, val, b, args, flops)
        cpu = None
        if not args.no_cpu_baseline:
            run, kind = cpu_arm_runner(m, val)
            times, xc = time_cpu(run, b, args.cpu_seconds)
            tmed = statistics.median(times)
            cpu = {"value": flops / tmed / 1e9, "unit": "GFLOP/s", "cores": 1, "kind": kind,
                   "sample": f"{len(times)} full serial solves of the {args.workload} matrix in {sum(times):.1f} s "
                             "(median; sptrsv_syncfree_executor FORWARD, transpose excluded)"}
            rel = float(np.max(np.abs(xh - xc)) / np.max(np.abs(xc)))
        else:
            rel = None
        info = solver.info()
        line = {
            "metric": "SpTRSV GFLOP/s (2*nnz-n flops per solve)", "value": value, "unit": "GFLOP/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
            "data": "synthetic (seeded generator, seed 0; stands in for the SuiteSparse set)",
            "config": {"workload": args.workload, "n": m.n, "nnz": m.nnz, "rhs": 1,
                       "algorithm": {1: "wrtfst", 2: "twopart", 3: "mix"}.get(info["algorithm"], "auto"),
                       "rows_per_thread": info["rows_per_thread"], "block": info["block_threads"],
                       "l2": "flushed between steps (512 MiB write outside the timed events); "
                             "inputs also exceed L2",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "row_solve_kernel", "kernel_ms": kms,
                         "algorithmic_bytes_per_launch": alg_bytes},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": 2 * args.steps,
            "gflops_2nnz": world * 2.0 * m.nnz / (ms * 1e-3) / 1e9,
            "gbs_algorithmic": alg_bytes / (ms * 1e-3) / 1e9,
            "rel_err_vs_cpu_reference": rel, "max_abs_x_minus_ones": max_dev,
            "wall_s_timed_region": t_wall,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def e2e_measure(cs, m, val, b, args, flops):
    """Same metric through the host-buffer C-ABI call: pinned b in, x out, per step."""
    import torch
    solver = cs.TriangularSolver(m.rowptr, m.colidx, val)  # host arrays: uploaded once at analysis
    bh = torch.from_numpy(np.ascontiguousarray(b)).pin_memory()
    xh = torch.empty_like(bh).pin_memory()
    bn, xn = bh.numpy(), xh.numpy()
    for _ in range(max(2, args.warmup)):
        solver.solve_host(bn, xn)
    reps = max(10, min(args.steps, 100))
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        solver.solve_host(bn, xn)
        times.append(time.perf_counter() - t0)
    sec = sum(times) / len(times)
    nbytes = b.nbytes
    # one-shot: analysis (upload + structure check + 1/diag) included
    t0 = time.perf_counter()
    s2 = cs.TriangularSolver(m.rowptr, m.colidx, val)
    s2.solve_host(bn, xn)
    first = time.perf_counter() - t0
    s2.close()
    solver.close()
    return {"value": flops / sec / 1e9, "unit": "GFLOP/s", "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes, "ms_per_step": sec * 1e3,
            "first_call_with_analysis_ms": first * 1e3}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in ("batched", "autograd"):
        from capellinisptrsv_gb300 import forms_bench
        return forms_bench.run(args)
    return run_native(args)


if __name__ == "__main__":
    sys.exit(main())
