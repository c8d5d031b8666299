"""Benchmark of the sync-free sparse triangular solve on GB300.

Default workload (N=1): the plain FP64 solve of the 4,194,304-row wide-level
matrix (1-7 off-diagonals per row in a band of 65,536; b = L*ones), the
configuration the headline metric is quoted on.  One step = one complete
solve (fill of x + the solve kernel) over inputs already resident in HBM.
The same JSON line also carries the two forms, each measured against its
per-system loop of plain solves (`forms`): the batched form (2,048 systems,
k = 1 and 16 right-hand sides, one CUDA-graph replay per step) and the
differentiation form (grad_1m, 16 RHS, forward + backward per step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]
                  [--workload wide_4m|plain_20k|zipf_1m|grad_1m|batched|autograd]
                  [--dtype f64|f32] [--no-forms]

Output: one JSON line on rank 0.  `value` is GFLOP/s with (2*nnz - n) flops
per solve (the benchmark definition's convention); `roofline` relates the
solve kernel's algorithmic bytes (4(n+1) + 4nnz + 4n + s*nnz + 2*s*n, the
reference's formula in CUDA/ourWrtFst/spts_syncfree_cuda_csr_wrt.h:208) per
launch to its CUDA-event duration, and the kernel time to its dependency-chain
floor (levels x the measured per-level hop); `e2e` is the same metric through
the host-buffer C-ABI call (capsp_solve_host: b read from pinned host memory,
x copied back); `cpu_baseline` is the reference's serial executor on the host
cores.  --impl reference times the reference's own CPU implementation instead;
that arm builds its inputs with the oracle library alone (the same seeded
generator, compiled into oracle/_build/liboracle.so) and never loads the
solver library.
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
    ap.add_argument("--no-vendor", action="store_true", help="skip the cuSPARSE SpSV side-by-side")
    ap.add_argument("--nsys", type=int, default=0, help="systems in the batched workload (default 2,048)")
    ap.add_argument("--no-forms", action="store_true", help="headline line without the batched/autograd forms")
    ap.add_argument("--forms-cpu-seconds", type=float, default=5.0, help="CPU baseline sample of each form")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(values, device):
    """Element-wise maximum over all ranks (the slowest replica sets the time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def replica_value(world: int, flops_per_solve: float, max_ms: float) -> float:
    """Whole-job GFLOP/s of N independent replicas: every rank solves once per step."""
    return world * flops_per_solve / (max_ms * 1e-3) / 1e9


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


def cpu_arm_runner(rowptr, colidx, val):
    """The reference's serial executor (oracle/_ref when built here, else the oracle port)."""
    import oracle
    ref = oracle.ref()
    if ref is not None:
        return ref.prepared_forward(rowptr, colidx, val), "reference"
    return oracle.prepared_forward(rowptr, colidx, val), "port"


def serial_sample(run, b, solves: int, warmup: int):
    """Per-solve wall times of `solves` full serial solves after `warmup` untimed
    ones.  Both CPU legs (the reference arm and the native line's cpu_baseline)
    use this, and both report the median."""
    x = np.empty_like(b)
    for _ in range(warmup):
        run(b, x)
    times = []
    for _ in range(solves):
        t0 = time.perf_counter()
        run(b, x)
        times.append(time.perf_counter() - t0)
    return times, x


def cpu_solves(args) -> int:
    """Serial solves per CPU measurement: the timed steps, at least 20."""
    return max(args.steps, 20)


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU implementation of the path, on inputs the
# oracle library generates (the solver library is never loaded here)
# ---------------------------------------------------------------------------

def oracle_workload(name: str, dtype):
    import oracle
    n, rp, ci, v = oracle.generate(name, seed=0)
    v = v.astype(dtype)
    return n, rp, ci, v, oracle.get_x_b(rp, v)


def oracle_batch_rhs(n, k):
    import oracle
    return oracle.normal(n * k, seed=0, stream=1000 + k).reshape(n, k)


def run_reference_forms(args):
    """Reference serial executor on the batched / autograd workloads (bounded samples per step)."""
    import oracle
    W = oracle.workloads()
    if args.workload == "batched":
        k = args.nrhs or BATCH_KS[0]
        n, rp, ci, v, so = oracle.generate_batched(args.nsys or BATCH_NSYS, seed=0)
        nsys = len(so) - 1
        picks = sorted(set(np.linspace(0, nsys - 1, 64).round().astype(int).tolist()))
        rhs = oracle_batch_rhs(n, k)
        work = []
        for s in picks:
            r0, r1, srp, sci, sv = W.sub_system(rp, ci, v, so, s)
            run, kind = cpu_arm_runner(srp, sci, sv)
            b = np.ascontiguousarray(rhs[r0:r1]) if k > 1 else rhs[r0:r1, 0].copy()
            work.append((run, b, np.empty_like(b)))
        # the systems are independent: one per host thread
        from concurrent.futures import ThreadPoolExecutor
        cores = host_threads()
        pool = ThreadPoolExecutor(cores)

        def one():
            _run_all(pool, work)
        per_step, unit = len(work) * k, "solves/s"
        metric = f"batched solves/s ({nsys} systems x k RHS)"
        sample = f"{len(work)} evenly spaced systems of {nsys} x {k} RHS per step, one system per host thread"
        steps = args.steps
        hib = True
    else:
        cores = 1  # one system: the executor takes all RHS in one serial call
        k = args.nrhs or AUTOGRAD_RHS
        n, rp, ci, v = oracle.generate("grad_1m", seed=0)
        b_h = oracle.normal(n * k, seed=0, stream=1).reshape(n, k)
        xs_h = oracle.normal(n * k, seed=0, stream=2).reshape(n, k)
        run, kind = cpu_arm_runner(rp, ci, v)
        adjoint = (oracle.ref() or oracle).solve_csr_transpose

        def one():
            x = run(b_h, np.empty_like(b_h))
            y = adjoint(rp, ci, v, x - xs_h)
            oracle.grad_val(rp, ci, y, x)
        per_step, unit = None, "ms"
        metric = f"fwd+bwd ms ({k} RHS)"
        sample = f"full grad_1m fwd+bwd with {k} RHS per step (steps capped at 10)"
        steps = min(args.steps, 10)
        hib = False
    for _ in range(min(args.warmup, 3)):
        one()
    t = []
    for _ in range(steps):
        t0 = time.perf_counter()
        one()
        t.append(time.perf_counter() - t0)
    sec = statistics.median(t)
    value = per_step / sec if per_step else sec * 1e3
    line = {
        "impl": "reference", "metric": metric, "value": value, "unit": unit, "n_gpus": args.gpus, "gpus_used": 0,
        "steps": steps,
        "warmup": min(args.warmup, 3), "ms_per_step": sec * 1e3, "higher_is_better": hib, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator, seed 0)",
        "config": {"workload": args.workload, "rhs": k},
        "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "host_cores": os.cpu_count(), "kind": kind,
                         "sample": sample + " (median step)"},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    if args.workload in ("batched", "autograd"):
        return run_reference_forms(args)
    dt = np.float64 if args.dtype == "f64" else np.float32
    n, rp, ci, val, b = oracle_workload(args.workload, dt)
    nnz = int(rp[-1])
    run, kind = cpu_arm_runner(rp, ci, val)
    steps, _ = serial_sample(run, b, args.steps, args.warmup)
    flops = 2.0 * nnz - n
    sec = statistics.median(steps)
    val_gf = flops / sec / 1e9
    line = {
        "impl": "reference", "metric": "SpTRSV GFLOP/s (2*nnz-n flops per solve)", "value": val_gf,
        "unit": "GFLOP/s", "n_gpus": args.gpus, "gpus_used": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": args.dtype, "data": "synthetic (seeded generator, seed 0)",
        "config": {"workload": args.workload, "n": n, "nnz": nnz, "rhs": 1,
                   "l2": "host run; inputs larger than the last-level cache"},
        "cpu_baseline": {"value": val_gf, "unit": "GFLOP/s", "cores": 1, "host_cores": os.cpu_count(), "kind": kind,
                         "sample": f"{args.steps} full serial solves of the {args.workload} matrix after "
                                   f"{args.warmup} untimed (median; sptrsv_syncfree_executor FORWARD; transpose "
                                   "and in-degree analysis excluded)",
                         "mean_ms": statistics.mean(steps) * 1e3},
        "e2e": {"value": val_gf, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gflops_2nnz": 2.0 * nnz / sec / 1e9,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# native arm
# ---------------------------------------------------------------------------

def run_native(args):
    world, rank, local = dist_env()
    dt = np.float64 if args.dtype == "f64" else np.float32
    s_bytes = 8 if dt == np.float64 else 4
    m, val, b = workload_matrix(args.workload, dt)
    flops = 2.0 * m.nnz - m.n
    # CPU baseline first, before this process initialises CUDA, with the same
    # procedure and estimator as the reference arm (median of the same solves)
    cpu, xc = None, None
    if rank == 0 and not args.no_cpu_baseline:
        run, kind = cpu_arm_runner(m.rowptr, m.colidx, val)
        times, xc = serial_sample(run, b, cpu_solves(args), args.warmup)
        tmed = statistics.median(times)
        cpu = {"value": flops / tmed / 1e9, "unit": "GFLOP/s", "cores": 1, "host_cores": os.cpu_count(),
               "kind": kind, "mean_ms": statistics.mean(times) * 1e3,
               "sample": f"{len(times)} full serial solves of the {args.workload} matrix after {args.warmup} untimed "
                         f"({sum(times):.1f} s; median; sptrsv_syncfree_executor FORWARD, transpose excluded)"}

    import torch
    import capellinisptrsv_gb300 as cs
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
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
        ms, kms = max_over_ranks([ms, kms], dev)

    # correctness spot-check against the reference's self-check (x_ref = ones)
    xh = x_d.cpu().numpy()
    max_dev = float(np.max(np.abs(xh - 1.0)))

    value = replica_value(world, flops, ms)
    alg_bytes = algorithmic_bytes(m.n, m.nnz, s_bytes)
    peak, peak_kind = peaks()
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    traffic = profile_traffic("row_solve", args.workload + "_" + args.dtype)
    info = solver.info()
    # dependency-chain floor: a solve of L levels takes at least L - 1 hops,
    # each costing at least one publication's detection on another warp
    hop_ns = cs.hop_latency(n=262_144, stride=64, dtype=dt)
    floor_ms = max(info["levels"] - 1, 0) * hop_ns * 1e-6

    line = None
    if rank == 0:
        e2e = None
        if not args.no_e2e:
            e2e = e2e_measure(cs, m, val, b, args, flops)
        vendor = None if args.no_vendor else vendor_measure(m, rp_d, ci_d, val_d, b_d, args, flops, kms)
        rel = float(np.max(np.abs(xh - xc)) / np.max(np.abs(xc))) if xc is not None else None
        line = {
            "metric": "SpTRSV GFLOP/s (2*nnz-n flops per solve)", "value": value, "unit": "GFLOP/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
            "data": "synthetic (seeded generator, seed 0; stands in for the SuiteSparse set)",
            "config": {"workload": args.workload, "n": m.n, "nnz": m.nnz, "rhs": 1, "levels": info["levels"],
                       "algorithm": {1: "wrtfst", 2: "twopart", 3: "mix"}.get(info["algorithm"], "auto"),
                       "rows_per_thread": info["rows_per_thread"], "block": info["block_threads"],
                       "l2": "flushed between steps (512 MiB write outside the timed events); "
                             "inputs also exceed L2",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "row_solve_kernel", "kernel_ms": kms,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "hop_ns": hop_ns, "latency_floor_ms": floor_ms,
                         "frac_of_floor": floor_ms / kms if kms > 0 else None,
                         "floor_how": "(levels - 1) x the per-level time of a chain matrix whose levels are "
                                      "64 rows in two warps, each row waiting on one row of the level before "
                                      "(capsp_hop_latency, n=262,144, stride 64, same dtype), measured live"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "cusparse_spsv": vendor,
            "gpu_launches": 2 * args.steps,
            "gflops_2nnz": world * 2.0 * m.nnz / (ms * 1e-3) / 1e9,
            "gbs_algorithmic": alg_bytes / (ms * 1e-3) / 1e9,
            "rel_err_vs_cpu_reference": rel, "max_abs_x_minus_ones": max_dev,
            "wall_s_timed_region": t_wall,
            "clocks": clk.summary(),
        }
    solver.close()
    del rp_d, ci_d, val_d, b_d, x_d, flush
    if rank == 0 and world == 1 and not args.no_forms and args.workload == "wide_4m":
        torch.cuda.empty_cache()
        try:
            line["forms"] = measure_forms(args)
        except Exception as e:  # the headline stands on its own: report the forms' failure in the line
            line["forms"] = {"error": f"{type(e).__name__}: {e}"[:500]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def vendor_measure(m, rp_d, ci_d, val_d, b_d, args, flops, capsp_kernel_ms):
    """cuSPARSE SpSV on the same device arrays: measured side-by-side, not a baseline of the metric."""
    import ctypes as C
    import torch
    lib_path = ROOT / "capellinisptrsv_gb300" / "_build" / "libcapsp_vendor.so"
    if not lib_path.exists():
        return {"unavailable": "libcapsp_vendor.so was not built"}
    lib = C.CDLL(str(lib_path))
    lib.capsp_vendor_spsv.restype = C.c_int
    lib.capsp_vendor_spsv.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    lib.capsp_vendor_last_error.restype = C.c_char_p
    x = torch.empty_like(b_d)
    an, so = C.c_float(), C.c_float()
    reps = max(3, min(args.steps, 20))
    torch.cuda.synchronize()
    rc = lib.capsp_vendor_spsv(m.n, m.nnz, rp_d.data_ptr(), ci_d.data_ptr(), val_d.data_ptr(),
                               0 if args.dtype == "f64" else 1, b_d.data_ptr(), x.data_ptr(), reps,
                               C.byref(an), C.byref(so))
    if rc != 0:
        return {"unavailable": lib.capsp_vendor_last_error().decode()}
    err = float((x.double() - 1.0).abs().max())
    return {"solve_ms": so.value, "value": flops / (so.value * 1e-3) / 1e9, "unit": "GFLOP/s",
            "analysis_ms": an.value, "solves_timed": reps, "max_abs_x_minus_ones": err,
            "capsp_kernel_speedup": so.value / capsp_kernel_ms,
            "what": "cusparseSpSV_solve (CUSPARSE_SPSV_ALG_DEFAULT, lower, non-unit) on the same device CSR "
                    "arrays, back-to-back solves after analysis; CUDA events"}


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
            "first_call_with_analysis_ms": first * 1e3,
            "how": "capsp_solve_host on pinned buffers: b goes up in doubling segments on a copy stream while "
                   "the solve runs (each chunk of rows waits for its segment's flag), and each 1/32 of x comes "
                   "back as soon as the kernel has counted all its rows finished"}


# ---------------------------------------------------------------------------
# the two forms: batched systems and differentiation
# ---------------------------------------------------------------------------
#
# batched:  2,048 independent systems, n log-uniform in [500, 50,000], 3-12
#           off-diagonals per row in a band of n/8 (seed 0), k right-hand sides
#           of N(0,1) values.  One step = one CUDA-graph replay of the
#           block-diagonal handle (launch shape picked by capsp_autotune).
#           Loop arm: one single-RHS capsp_solve per system and RHS column, each
#           system on its own handle (a bounded, evenly spaced sample of
#           systems per step).  Metric: solves/s = systems x k / time.
# autograd: grad_1m (n=1,048,576, 2-10 off-diagonals in a band of 16,384),
#           16 RHS of N(0,1), target x* ~ N(0,1), loss 0.5*||x - x*||^2.
#           One step = forward + backward through SparseTriangularSolve.
#           Loop arm: 16 single-RHS forward solves + 16 single-RHS solves of the
#           explicitly transposed (upper CSR) matrix + one grad_val pass.
#           Metric: fwd+bwd ms.

BATCH_NSYS = 2048
BATCH_KS = (1, 4, 16, 32)
LOOP_SOLVES_PER_STEP = 2048
AUTOGRAD_RHS = 16


def _sub_system(m, s):
    """Rows [r0, r1) of system s as a standalone CSR (indices rebased)."""
    from capellinisptrsv_gb300 import workloads as W
    return W.sub_system(m.rowptr, m.colidx, m.val, m.sys_rowoff, s)


def _single_gpu_forms(args):
    world, _, _ = dist_env()
    if world > 1:
        raise SystemExit("the batched and autograd workloads run on one GPU (use --gpus 1)")


def _batch_rhs(cs, n, k):
    return cs.normal(n * k, seed=0, stream=1000 + k).reshape(n, k)


def host_threads() -> int:
    """Host cores this process may run on."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


def _run_all(pool, work):
    """Run (run, b, x) items concurrently: the executors are C calls that release the GIL."""
    for f in [pool.submit(run, b, x) for run, b, x in work]:
        f.result()


def _cpu_batched(cs, m, k, seconds):
    """Reference serial executor, one system per host thread (the systems are
    independent; each group is prepared outside the clock).  Returns the rate
    and the solutions of the systems it solved, (r0, r1, x) each."""
    from concurrent.futures import ThreadPoolExecutor
    threads = host_threads()
    rhs = _batch_rhs(cs, m.n, k)
    nsys = len(m.sys_rowoff) - 1
    run_kind = None
    solved, spent, systems, s = 0, 0.0, 0, 0
    sols = []
    with ThreadPoolExecutor(threads) as pool:
        while s < nsys and spent < seconds:
            work, rows = [], []
            for _ in range(4 * threads):
                if s >= nsys:
                    break
                r0, r1, rp, ci, v = _sub_system(m, s)
                run, run_kind = cpu_arm_runner(rp, ci, v)
                b = np.ascontiguousarray(rhs[r0:r1]) if k > 1 else rhs[r0:r1, 0].copy()
                work.append((run, b, np.empty_like(b)))
                rows.append((r0, r1))
                s += 1
            t0 = time.perf_counter()
            _run_all(pool, work)
            spent += time.perf_counter() - t0
            solved += len(work) * k
            systems += len(work)
            sols.extend((r0, r1, w[2]) for (r0, r1), w in zip(rows, work))
    return solved / spent, run_kind, systems, spent, threads, sols


def _rel(a, r) -> float:
    a, r = np.asarray(a, np.float64), np.asarray(r, np.float64)
    return float(np.max(np.abs(a - r)) / max(np.max(np.abs(r)), 1e-300))


def measure_batched(args, ks, cpu_seconds, e2e: bool = True):
    """The batched form on one GPU: per k, one CUDA-graph replay per step
    against a loop of single-RHS plain solves; the CPU baseline (and the
    result check against it) and e2e at the first k."""
    import ctypes as C
    import torch
    import capellinisptrsv_gb300 as cs
    from capellinisptrsv_gb300 import _native as N
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    m = cs.generate_batched(args.nsys or BATCH_NSYS, seed=0)
    nsys = len(m.sys_rowoff) - 1
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    rp_d, ci_d, val_d = to(m.rowptr), to(m.colidx), to(m.val)
    t0 = time.perf_counter()
    batch = cs.TriangularSolver(rp_d, ci_d, val_d, sys_rowoff=m.sys_rowoff)
    analyse_s = time.perf_counter() - t0
    st = torch.cuda.Stream(dev)
    sth = C.c_void_p(st.cuda_stream)

    # one handle per system for the loop arm (host arrays, uploaded at analysis)
    handles = {}

    def handle(s):
        if s not in handles:
            r0, r1, rp, ci, v = _sub_system(m, s)
            handles[s] = (r0, r1, cs.TriangularSolver(rp, ci, v))
        return handles[s]

    peak, peak_kind = peaks()
    sweep = []
    x_first = None
    for k in ks:
        b_h = _batch_rhs(cs, m.n, k)
        b_d = to(b_h if k > 1 else b_h[:, 0])
        x_d = torch.empty_like(b_d)
        with torch.cuda.stream(st):
            tune_ms = batch.autotune(b_d, x_d, stream=st)
            for _ in range(max(3, args.warmup)):
                batch.graph_solve(b_d, x_d, st)
        st.synchronize()
        batch.status(st)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with ClockSampler(0) as clk:
            for i in range(args.steps):
                ev[i][0].record(st)
                batch.graph_solve(b_d, x_d, st)
                ev[i][1].record(st)
            st.synchronize()
        batch.status(st)
        ms = statistics.mean(a.elapsed_time(bb) for a, bb in ev)
        # kernel time of the same launch shape, plain launches with profiling on
        batch.set_profiling(True)
        kms = []
        for _ in range(3):
            batch.solve(b_d, x_d, stream=st)
            kms.append(batch.last_kernel_ms())
        batch.set_profiling(False)
        kms = statistics.mean(kms)
        info = batch.info()

        # loop arm: a bounded, evenly spaced sample of systems, every RHS column
        nloop = max(1, min(nsys, LOOP_SOLVES_PER_STEP // k))
        picks = sorted(set(np.linspace(0, nsys - 1, nloop).round().astype(int).tolist()))
        cols = []
        for s in picks:
            r0, r1, hs = handle(s)
            for j in range(k):
                bc = b_d[r0:r1, j].contiguous() if k > 1 else b_d[r0:r1].contiguous()
                cols.append((hs._h, bc, torch.empty_like(bc)))
        fn = N.lib.capsp_solve
        calls = [(h, C.c_void_p(bc.data_ptr()), C.c_void_p(xc.data_ptr())) for h, bc, xc in cols]

        def loop_pass():
            for h, pb, px in calls:
                N.check(fn(h, pb, px, 1, 1, sth))

        with torch.cuda.stream(st):
            loop_pass()
            st.synchronize()
            loop_steps = max(1, min(args.steps, 3))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(loop_steps):
                loop_pass()
            e1.record(st)
            st.synchronize()
        loop_ms = e0.elapsed_time(e1) / loop_steps
        # the loop's results against the batched launch's
        xb = x_d.cpu().numpy().reshape(m.n, -1)
        if x_first is None:
            x_first = xb
        worst, c = 0.0, 0
        for s in picks:
            r0, r1, _ = handles[s]
            for j in range(k):
                worst = max(worst, _rel(cols[c][2].cpu().numpy(), xb[r0:r1, j]))
                c += 1
        solves = nsys * k
        entry = {
            "k": k, "solves_per_s": solves / (ms * 1e-3), "ms_per_step": ms, "kernel_ms": kms,
            "loop_solves_per_s": len(calls) / (loop_ms * 1e-3), "loop_solves_per_step": len(calls),
            "loop_systems": len(picks), "loop_ms_per_step": loop_ms,
            "rows_per_thread": info["rows_per_thread"], "block": info["block_threads"],
            "blocks_per_sm": info["blocks_per_sm"], "autotune_best_ms": tune_ms,
            "loop_vs_batched_rel_err": worst, "clocks": clk.summary(),
        }
        entry["speedup_vs_loop"] = entry["solves_per_s"] / entry["loop_solves_per_s"]
        alg = algorithmic_bytes(m.n, m.nnz, 8, k)
        # DRAM bytes per launch from a committed capture of this k (default batch)
        traffic = profile_traffic("row_solve", f"batched_k{k}_f64") if nsys == BATCH_NSYS else None
        entry["roofline"] = {"bound": "hbm", "achieved": alg / (kms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                             "frac": alg / (kms * 1e-3) / 1e9 / peak, "traffic": traffic, "peak_kind": peak_kind,
                             "kernel": "row_solve_kernel", "kernel_ms": kms, "algorithmic_bytes_per_launch": alg}
        sweep.append(entry)
        del b_d, x_d, cols, calls

    k = ks[0]
    out = {"nsys": nsys, "n": m.n, "nnz": m.nnz, "levels": batch.info()["levels"], "analyse_s": analyse_s,
           "sweep": sweep}
    if e2e:
        # end to end through the host-buffer call: pinned b in, x out, every step
        b_h = _batch_rhs(cs, m.n, k)
        b_h = b_h if k > 1 else b_h[:, 0].copy()
        bh = torch.from_numpy(np.ascontiguousarray(b_h)).pin_memory()
        xh = torch.empty_like(bh).pin_memory()
        batch.solve_host(bh.numpy(), xh.numpy())
        reps = max(3, min(args.steps, 20))
        t0 = time.perf_counter()
        for _ in range(reps):
            batch.solve_host(bh.numpy(), xh.numpy())
        e2e_s = (time.perf_counter() - t0) / reps
        out["e2e"] = {"value": nsys * k / e2e_s, "unit": "solves/s", "rhs": k,
                      "h2d_bytes_per_step": int(bh.numel() * 8), "d2h_bytes_per_step": int(xh.numel() * 8),
                      "ms_per_step": e2e_s * 1e3}
    out["cpu_baseline"] = None
    if cpu_seconds > 0:
        v, kind, systems, spent, threads, sols = _cpu_batched(cs, m, k, cpu_seconds)
        out["cpu_baseline"] = {
            "value": v, "unit": "solves/s", "rhs": k, "cores": threads, "host_cores": os.cpu_count(), "kind": kind,
            "sample": f"first {systems} of {nsys} systems x {k} RHS in {spent:.1f} s, one system per host "
                      f"thread on {threads} threads (sptrsv_syncfree_executor FORWARD; transpose and "
                      "analysis excluded)"}
        # the batched GPU result against the serial executor's, system by system
        out["rel_err_vs_cpu_reference"] = max(_rel(x_first[r0:r1].reshape(r1 - r0, -1), xs.reshape(r1 - r0, -1))
                                             for r0, r1, xs in sols)
        out["systems_checked_vs_cpu_reference"] = len(sols)
    batch.close()
    for _, _, hs in handles.values():
        hs.close()
    return out


def run_batched(args):
    _single_gpu_forms(args)
    ks = [args.nrhs] if args.nrhs else list(BATCH_KS)
    d = measure_batched(args, ks, 0.0 if args.no_cpu_baseline else args.cpu_seconds)
    head = d["sweep"][0]
    k = head["k"]
    line = {
        "metric": f"batched solves/s ({d['nsys']} systems x k RHS)", "value": head["solves_per_s"],
        "unit": "solves/s", "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded generator, seed 0)",
        "config": {"workload": "batched", "nsys": d["nsys"], "n": d["n"], "nnz": d["nnz"], "rhs": k,
                   "levels": d["levels"],
                   "launch": "CUDA graph replay of one persistent solve (autotuned launch shape)",
                   "l2": f"inputs ({algorithmic_bytes(d['n'], d['nnz'], 8, k) / 1e9:.1f} GB) larger than L2, "
                         "no flush",
                   "parallelism": "single GPU"},
        "roofline": head["roofline"], "cpu_baseline": d["cpu_baseline"], "e2e": d["e2e"],
        "gpu_launches": 2 * args.steps,
        "loop_baseline": {"value": head["loop_solves_per_s"], "unit": "solves/s",
                          "what": "one single-RHS capsp_solve per system and RHS column, each system on its own "
                                  "handle, on an evenly spaced sample of systems"},
        "speedup_vs_loop": head["speedup_vs_loop"], "sweep": d["sweep"], "clocks": head["clocks"],
        "rel_err_vs_cpu_reference": d.get("rel_err_vs_cpu_reference"),
    }
    print(json.dumps(line), flush=True)
    return 0


def _grad_bytes(n, nnz, s, k):
    """grad_val pass: rowptr, colidx, y and x (each row once), grad_val written."""
    return 4.0 * (n + 1) + 4.0 * nnz + 2.0 * s * n * k + s * nnz


def measure_autograd(args, cpu_seconds):
    """The differentiation form: forward + backward through SparseTriangularSolve
    against a loop of single-RHS solves; CPU fwd+bwd and the result check against it."""
    import torch
    import capellinisptrsv_gb300 as cs
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    k = args.nrhs if (args.nrhs and args.workload == "autograd") else AUTOGRAD_RHS
    m = cs.generate("grad_1m", seed=0)
    n = m.n
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    rp_d, ci_d = to(m.rowptr), to(m.colidx)
    val = to(m.val).requires_grad_(True)
    b_h = cs.normal(n * k, seed=0, stream=1).reshape(n, k)
    xs_h = cs.normal(n * k, seed=0, stream=2).reshape(n, k)
    b = to(b_h).requires_grad_(True)
    xstar = to(xs_h)
    solver = cs.TriangularSolver(rp_d, ci_d, val.detach())
    stream = torch.cuda.current_stream(dev)

    def step():
        val.grad = None
        b.grad = None
        x = cs.sptrsv(solver, val, b)
        loss = 0.5 * ((x - xstar) ** 2).sum()
        loss.backward()
        return loss

    for _ in range(max(3, args.warmup)):
        step()
    solver.status()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(0) as clk:
        for i in range(args.steps):
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    solver.status()
    ms = statistics.mean(a.elapsed_time(bb) for a, bb in ev)
    g_val, g_b = val.grad.clone(), b.grad.clone()

    # kernel times: forward row solve, the transposed view's row solve, the
    # grad_val pass (CUDA events on the launching stream around it alone)
    solver.set_profiling(True)
    x = solver.solve(b.detach())
    kf = solver.last_kernel_ms()
    gx = (x - xstar).contiguous()
    y = solver.solve_transpose(gx)
    kt = solver.last_kernel_ms()
    solver.set_profiling(False)
    gv_out = torch.empty(m.nnz, dtype=torch.float64, device=dev)
    solver.grad_val(y, x, out=gv_out)
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    g0.record(stream)
    for _ in range(5):
        solver.grad_val(y, x, out=gv_out)
    g1.record(stream)
    torch.cuda.synchronize()
    kg = g0.elapsed_time(g1) / 5
    x_gpu = x.cpu().numpy()

    # loop arm: single-RHS solves of L and of an explicitly transposed L
    cp, ri, cv = cs.matrix_transposition(n, n, m.nnz, m.rowptr, m.colidx, m.val)
    upper = cs.TriangularSolver(to(cp), to(ri), to(cv), uplo="upper")
    bcols = [b.detach()[:, j].contiguous() for j in range(k)]
    xscols = [xstar[:, j].contiguous() for j in range(k)]

    def loop_step():
        xs = [solver.solve(bc) for bc in bcols]
        gs = [xc - xsc for xc, xsc in zip(xs, xscols)]
        loss = 0.5 * sum((gc ** 2).sum() for gc in gs)
        ys = [upper.solve(gc) for gc in gs]
        y, xm = torch.stack(ys, dim=1), torch.stack(xs, dim=1)
        return loss, y, solver.grad_val(y, xm)

    for _ in range(2):
        loop_step()
    loop_steps = max(1, min(args.steps, 10))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(loop_steps):
        _, y_loop, gv_loop = loop_step()
    e1.record(stream)
    torch.cuda.synchronize()
    loop_ms = e0.elapsed_time(e1) / loop_steps
    upper.status()
    rel = lambda a, r: float((a - r).abs().max() / r.abs().max())
    agree = {"grad_b": rel(g_b, y_loop), "grad_val": rel(g_val, gv_loop)}

    # end to end: host b and x* copied in, loss read back, every step
    bh = torch.from_numpy(b_h).pin_memory()
    xsh = torch.from_numpy(xs_h).pin_memory()

    def e2e_step():
        b_in = bh.to(dev, non_blocking=True).requires_grad_(True)
        xs_in = xsh.to(dev, non_blocking=True)
        val.grad = None
        x = cs.sptrsv(solver, val, b_in)
        loss = 0.5 * ((x - xs_in) ** 2).sum()
        loss.backward()
        return float(loss.detach())

    e2e_step()
    reps = max(3, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(reps):
        e2e_step()
    e2e_ms = (time.perf_counter() - t0) / reps * 1e3

    peak, peak_kind = peaks()
    fwd_bytes = algorithmic_bytes(n, m.nnz, 8, k)
    grad_bytes = _grad_bytes(n, m.nnz, 8, k)
    kernels = {
        "forward_row_solve": {"kernel": "row_solve_kernel", "kernel_ms": kf, "algorithmic_bytes_per_launch": fwd_bytes,
                              "achieved": fwd_bytes / (kf * 1e-3) / 1e9,
                              "traffic": profile_traffic("row_solve", f"grad_1m_{k}rhs_f64")},
        "transpose_row_solve": {"kernel": "row_solve_kernel over the transposed view", "kernel_ms": kt,
                                "algorithmic_bytes_per_launch": fwd_bytes,
                                "achieved": fwd_bytes / (kt * 1e-3) / 1e9,
                                "traffic": profile_traffic("row_solve_transpose", f"grad_1m_{k}rhs_f64")},
        "grad_val": {"kernel": "grad_val_kernel", "kernel_ms": kg, "algorithmic_bytes_per_launch": grad_bytes,
                     "achieved": grad_bytes / (kg * 1e-3) / 1e9,
                     "fp64_fma_per_launch": float(m.nnz) * k,
                     "traffic": profile_traffic("grad_val", f"grad_1m_{k}rhs_f64")},
    }
    for r in kernels.values():
        r.update({"bound": "hbm", "peak": peak, "unit": "GB/s", "frac": r["achieved"] / peak, "peak_kind": peak_kind})
    roof = max(kernels.values(), key=lambda r: r["kernel_ms"])
    out = {"n": n, "nnz": m.nnz, "rhs": k, "ms_per_step": ms, "kernel_ms": {"forward_row_solve": kf,
                                                                              "transpose_row_solve": kt,
                                                                              "grad_val": kg},
           "roofline": roof, "kernels": kernels,
           "loop_baseline": {"value": loop_ms, "unit": "ms",
                             "what": f"{k} single-RHS solves of L + {k} single-RHS solves of an explicit L^T "
                                     "(upper CSR) + one grad_val pass"},
           "speedup_vs_loop": loop_ms / ms, "loop_vs_autograd_rel_err": agree, "clocks": clk.summary(),
           "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": int(2 * n * k * 8), "d2h_bytes_per_step": 8},
           # forward: 1/diag + the level values of both views (3), pending
           # fill, row solve; backward: pending fill, row solve over the
           # transposed view, grad_val (no refresh: the values are still bound)
           "gpu_launches_per_step": 8}
    out["cpu_baseline"] = None
    if cpu_seconds > 0:
        cpu, (xc, yc, gc) = _cpu_autograd(m, b_h, xs_h, cpu_seconds)
        out["cpu_baseline"] = cpu
        # the GPU gradients against the serial forward / adjoint / grad_val
        out["rel_err_vs_cpu_reference"] = {"x": _rel(x_gpu, xc), "grad_b": _rel(g_b.cpu().numpy(), yc),
                                           "grad_val": _rel(g_val.cpu().numpy(), gc)}
    solver.close()
    upper.close()
    return out


def run_autograd(args):
    _single_gpu_forms(args)
    d = measure_autograd(args, 0.0 if args.no_cpu_baseline else args.cpu_seconds)
    k = d["rhs"]
    line = {
        "metric": f"fwd+bwd ms ({k} RHS)", "value": d["ms_per_step"], "unit": "ms", "n_gpus": 1, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": d["ms_per_step"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator, seed 0)",
        "config": {"workload": "autograd", "matrix": "grad_1m", "n": d["n"], "nnz": d["nnz"], "rhs": k,
                   "loss": "0.5*||x - x*||^2",
                   "l2": "inputs (matrix, b, x, x*) larger than L2, no flush", "parallelism": "single GPU"},
        "roofline": d["roofline"], "cpu_baseline": d["cpu_baseline"], "e2e": d["e2e"],
        "gpu_launches": d["gpu_launches_per_step"] * args.steps,
        "kernel_ms": d["kernel_ms"], "kernels": d["kernels"], "loop_baseline": d["loop_baseline"],
        "speedup_vs_loop": d["speedup_vs_loop"], "loop_vs_autograd_rel_err": d["loop_vs_autograd_rel_err"],
        "rel_err_vs_cpu_reference": d.get("rel_err_vs_cpu_reference"), "clocks": d["clocks"],
    }
    print(json.dumps(line), flush=True)
    return 0


def _cpu_autograd(m, b_h, xs_h, seconds):
    """Serial forward (k RHS), serial adjoint (BACKWARD executor on L's CSR) and
    grad_val, median over passes; also returns the last pass's (x, y, grad_val)."""
    import oracle
    run, kind = cpu_arm_runner(m.rowptr, m.colidx, m.val)
    adjoint = (oracle.ref() or oracle).solve_csr_transpose
    times = []
    t_end = time.perf_counter() + seconds
    res = None
    while not times or time.perf_counter() < t_end:
        t0 = time.perf_counter()
        x = run(b_h, np.empty_like(b_h))
        y = adjoint(m.rowptr, m.colidx, m.val, x - xs_h)
        g = oracle.grad_val(m.rowptr, m.colidx, y, x)
        times.append(time.perf_counter() - t0)
        res = (x, y, g)
    return {"value": statistics.median(times) * 1e3, "unit": "ms", "cores": 1, "host_cores": os.cpu_count(),
            "kind": kind, "sample": f"{len(times)} serial fwd+bwd passes over the full grad_1m system with "
                                    f"{b_h.shape[1]} RHS (median)"}, res


FORMS_KS = (1, 16)


def measure_forms(args):
    """Both forms at their benchmark sizes, compacted for the headline line."""
    bt = measure_batched(args, FORMS_KS, args.forms_cpu_seconds, e2e=True)
    batched = {
        "metric": "solves/s", "nsys": bt["nsys"], "n": bt["n"], "nnz": bt["nnz"], "levels": bt["levels"],
        "launch": "CUDA graph replay of one persistent solve (autotuned launch shape)",
        "per_k": {str(e["k"]): {key: e[key] for key in ("solves_per_s", "ms_per_step", "kernel_ms",
                                                         "loop_solves_per_s", "speedup_vs_loop", "roofline",
                                                         "loop_vs_batched_rel_err", "clocks")}
                  for e in bt["sweep"]},
        "loop_what": "one single-RHS capsp_solve per system and RHS column, each system on its own handle, "
                     "on an evenly spaced sample of systems",
        "cpu_baseline": bt["cpu_baseline"], "e2e": bt.get("e2e"),
        "rel_err_vs_cpu_reference": bt.get("rel_err_vs_cpu_reference"),
        "systems_checked_vs_cpu_reference": bt.get("systems_checked_vs_cpu_reference"),
    }
    ag = measure_autograd(args, args.forms_cpu_seconds)
    autograd = {key: ag[key] for key in ("n", "nnz", "rhs", "ms_per_step", "kernel_ms", "kernels", "loop_baseline",
                                          "speedup_vs_loop", "loop_vs_autograd_rel_err", "cpu_baseline", "e2e",
                                          "clocks")}
    autograd["metric"] = "fwd+bwd ms"
    autograd["rel_err_vs_cpu_reference"] = ag.get("rel_err_vs_cpu_reference")
    return {"batched": batched, "autograd": autograd,
            "steps": args.steps, "warmup": max(3, args.warmup), "dtype": "f64"}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "autograd":
        return run_autograd(args)
    return run_native(args)


if __name__ == "__main__":
    sys.exit(main())
