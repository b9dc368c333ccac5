#!/usr/bin/env python
"""Headline benchmark: wall-Stokeslet kernel sum (fl.evaluate(WallStokeslet3D, ...)).

Workload (one step): 262,144 targets uniform in [-1,1]^2 x [0.02,2] plus 16,384
targets on the wall z = 0, 262,144 sources in the same box, i.i.d. N(0,1)
FP64 forces, eps = 0.01, seeded (synthetic, the reference publishes no
dataset).  One step = one mixed-precision sum (FP32 far field + FP64 near
field for r < 4 eps) over all 278,528 x 262,144 pairs; inputs resident in HBM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line.  Timing: CUDA events on the launching stream around each
step, L2 flushed (256 MB write) between timed steps, max over ranks; e2e goes
through the public API with pinned host buffers (H2D + D2H inside the timed
region).  The roofline of the dominant kernel (far_f32_kernel) uses the
per-launch durations recorded by the library's CUDA events and the FP32 FFMA
peak measured in the same process.  Multi-GPU: each rank sums its own
independent workload (weak scaling, no collective on the data path).
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

N_SRC, N_TGT, N_WALL, EPS = 262144, 262144, 16384, 0.01
FLOPS_PER_PAIR = 106          # WallStokeslet3D: canonical count (31 Stokeslet + 75 image)
METRIC = "pair-interactions/s"
WORKLOAD = "WallStokeslet3D sum, 278,528 targets (16,384 on z=0) x 262,144 sources, eps=0.01"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--cpu-sample", type=int, default=16384, help="targets in the CPU slice (x all sources)")
    p.add_argument("--cpu-chunk", type=int, default=2048,
                   help="targets of the CPU slice timed per step of --impl reference (the slice in turn)")
    p.add_argument("--no-extras", action="store_true", help="skip the accuracy / FP64 / solve sections")
    p.add_argument("--workload", default="wall_sum", choices=["wall_sum", "brinkman_gmres", "wall_lu", "serve"],
                   help="wall_sum (default, the headline) or one of the other benchmark configurations")
    p.add_argument("--n-points", type=int, default=None, help="override the point count of brinkman_gmres / wall_lu")
    p.add_argument("--fp64", action="store_true", help="also run the plain FP64 GPU solve (slow at full size)")
    p.add_argument("--slots", type=int, default=6, help="solve-server slots (serve workload)")
    p.add_argument("--rates", default="50,200,800", help="Poisson arrival rates (serve workload)")
    p.add_argument("--batch", type=int, default=4, help="most same-bucket requests per batched factorization "
                                                        "(serve workload)")
    # one hot-path operation at a chosen size, for profiler captures (no JSON line)
    p.add_argument("--case", default=None,
                   choices=["sum", "assemble", "lu", "resistance", "breakdown", "swim", "lu_batch"],
                   help="run one operation at a chosen size for a profiler capture instead of the benchmark")
    p.add_argument("--kind", default="wall", choices=["stokeslet", "wall", "brinkman"])
    p.add_argument("--alpha", type=complex, default=0.0)
    p.add_argument("--targets", type=int, default=65536)
    p.add_argument("--sources", type=int, default=262144)
    p.add_argument("--precision", default="mixed")
    p.add_argument("--n", type=int, default=1536, help="points for the assemble / lu / resistance cases")
    p.add_argument("--lu", default="tf32")
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--nbat", type=int, default=4, help="systems per group (lu_batch case)")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def ranks_throughput(dist, local_ms, units_per_rank, world, device=None, reduce="max"):
    """Whole-job throughput of `world` independent replicas: every rank processed
    units_per_rank units; the job took as long as the slowest rank (reduce="max" over the
    ranks' times; "min" over per-rank throughputs for the end-to-end figure).  Returns
    (units per second, the time in ms that it is based on)."""
    import torch

    if reduce == "max":
        t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        return units_per_rank * world / (ms * 1e-3), ms
    rate = torch.tensor([units_per_rank * world / (float(local_ms) * 1e-3)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(rate, op=dist.ReduceOp.MIN)
    r = float(rate.item())
    return r, units_per_rank * world / r * 1e3


def make_workload(seed):
    from fluidlets_gb300.geometry import wall_sum_workload

    return wall_sum_workload(N_SRC, N_TGT, N_WALL, EPS, seed=seed)


def cpu_slice(T, n_targets):
    """The CPU baseline's slice of the targets: n_targets of them, evenly strided over the set."""
    return T[:: max(1, len(T) // n_targets)][:n_targets]


def cpu_sample_rate(sub, S, F, eps):
    """The oracle (C/OpenMP restatement of the reference loop, -O3) on all host cores."""
    import oracle

    threads = oracle.max_threads()
    t0 = time.perf_counter()
    oracle.evaluate("wall", sub, S, F, eps)
    dt = time.perf_counter() - t0
    return len(sub) * len(S) / dt, threads


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    T, S, F, eps = make_workload(0)
    rates = []
    import oracle

    oracle.build()
    sl = cpu_slice(T, args.cpu_sample)
    nchunk = max(1, len(sl) // args.cpu_chunk)
    pairs = []
    for i in range(args.warmup + args.steps):
        c = i % nchunk
        sub = sl[c * args.cpu_chunk:(c + 1) * args.cpu_chunk]
        r, threads = cpu_sample_rate(sub, S, F, eps)
        if i >= args.warmup:
            rates.append(r)
            pairs.append(len(sub) * N_SRC)
    sample = (f"{len(sl)}-target slice (every {max(1, len(T) // args.cpu_sample)}th target) x {N_SRC} sources, "
              f"{args.cpu_chunk} targets of it per step in turn (WallStokeslet3D, FP64); pairs/s scale linearly "
              "to the full 278,528 x 262,144 sum")
    total_pairs = sum(pairs)
    total_time = sum(p / r for p, r in zip(pairs, rates))
    value = total_pairs / total_time
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_time / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def solve_section(dev, n_points=1536, reps=5):
    """Resistance solves on the sphere workload: unit sphere, N Fibonacci points, eps = 0.25 x mean
    nearest-neighbour spacing, U = (1, 0, 0), free-space Stokeslet, dense LU (3N unknowns).
    Plain FP64 GPU path vs mixed precision (tensor-core LU + FP64 GMRES-IR), with a cuSOLVER
    FP64 solve (torch.linalg.solve) of the same assembled matrix as a reference point."""
    import torch

    import fluidlets_gb300 as fl
    from fluidlets_gb300.core import _assemble_dev
    from fluidlets_gb300.geometry import fibonacci_sphere, mean_nn_spacing

    X = fibonacci_sphere(n_points)
    eps = 0.25 * mean_nn_spacing(X)
    Xd = torch.from_numpy(X).to(dev)
    U = torch.zeros_like(Xd)
    U[:, 0] = 1.0
    ed = torch.full((n_points,), eps, dtype=torch.float64, device=dev)
    kern = fl.Stokeslet3D()

    def timed(fn):
        out = fn()  # warm-up
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            ms.append(1e3 * (time.perf_counter() - t0))
        ms = np.array(ms)
        return out, {"solves_per_s": float(1e3 / ms.mean()), "ms_mean": float(ms.mean()),
                     "p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99))}

    (F64, i64), t64 = timed(lambda: fl.resistance(kern, Xd, U, ed, method="lu"))
    res = {"workload": f"resistance, free Stokeslet, unit sphere N={n_points} Fibonacci, eps={eps:.6f} "
                       f"(0.25 x mean NN spacing), U=(1,0,0), dense LU on {3 * n_points} unknowns",
           "fp64_gpu": dict(t64, residual=i64.residual),
           "drag_over_6pi_a": float(F64[:, 0].sum().item() / (6 * np.pi))}
    for lu in ("tf32", "bf16"):
        (Fm, im), tm = timed(lambda: fl.resistance(kern, Xd, U, ed, method="lu", precision="mixed", lu=lu))
        err = float(torch.linalg.vector_norm(Fm - F64) / torch.linalg.vector_norm(F64))
        res[f"mixed_{lu}"] = dict(tm, rel_force_err_vs_fp64=err, residual=im.residual, ir_steps=im.ir_steps,
                                  gmres_iterations=im.iterations, speedup_vs_fp64=t64["ms_mean"] / tm["ms_mean"])

    def cusolver():
        K = _assemble_dev(kern, Xd, Xd, ed, 1.0)
        return torch.linalg.solve(K, U.reshape(-1))

    try:  # a library reference point only (torch loads cuSOLVER lazily; it may be unavailable)
        _, tc = timed(cusolver)
    except RuntimeError as e:
        tc = {"unavailable": str(e).splitlines()[0][:200], "ms_mean": float("inf")}
    res["cusolver_fp64_reference_point"] = tc
    res["fp64_baseline_for_speedup"] = "fp64_gpu" if t64["ms_mean"] <= tc["ms_mean"] else "cusolver_fp64_reference_point"
    base = min(t64["ms_mean"], tc["ms_mean"])
    for lu in ("tf32", "bf16"):
        res[f"mixed_{lu}"]["speedup_vs_faster_fp64"] = base / res[f"mixed_{lu}"]["ms_mean"]
    return res


def wall_lu_section(dev, n_points=8192, h=1.05, reps=3):
    """Mixed-precision dense resistance near a wall: sphere radius 1, N Fibonacci points centred at
    h/a over z = 0, eps = 0.25 x mean NN spacing, WallStokeslet3D, translation parallel to the wall
    (3N unknowns); TF32 and BF16 tensor-core LU + FP64 GMRES-IR against one FP64 GPU LU."""
    import torch

    import fluidlets_gb300 as fl
    from fluidlets_gb300.geometry import fibonacci_sphere, mean_nn_spacing

    S = fibonacci_sphere(n_points)
    eps = 0.25 * mean_nn_spacing(S)
    X = torch.from_numpy(S + [0.0, 0.0, h]).to(dev)
    e = torch.full((n_points,), eps, dtype=torch.float64, device=dev)
    U = torch.zeros_like(X)
    U[:, 0] = 1.0
    k = fl.WallStokeslet3D()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    F64, i64 = fl.resistance(k, X, U, e, method="lu")
    torch.cuda.synchronize()
    res = {"workload": f"WallStokeslet3D resistance, sphere N={n_points} ({3 * n_points} unknowns) at h/a={h}, "
                       f"eps={eps:.7f}, translation parallel to the wall, dense LU",
           "fp64_gpu": {"ms": 1e3 * (time.perf_counter() - t0), "residual": i64.residual},
           "drag_x": float(F64[:, 0].sum())}
    for lu in ("tf32", "bf16"):
        fl.resistance(k, X, U, e, method="lu", precision="mixed", lu=lu)  # warm-up
        ms = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Fm, im = fl.resistance(k, X, U, e, method="lu", precision="mixed", lu=lu)
            torch.cuda.synchronize()
            ms.append(1e3 * (time.perf_counter() - t0))
        err = float(torch.linalg.vector_norm(Fm - F64) / torch.linalg.vector_norm(F64))
        res[f"mixed_{lu}"] = {"ms_mean": float(np.mean(ms)), "solves_per_s": float(1e3 / np.mean(ms)),
                              "rel_force_err_vs_fp64": err, "residual": im.residual, "ir_steps": im.ir_steps,
                              "gmres_iterations": im.iterations,
                              "speedup_vs_fp64": res["fp64_gpu"]["ms"] / float(np.mean(ms))}
        # the tensor-core trailing updates of one solve: 2/3 n^3 flops over their own launches' time
        # (CUDA events on the launching stream); the denominator is a cuBLAS GEMM of the same operand
        # type measured below
        from fluidlets_gb300 import _lib

        L = _lib.load()
        # one solve through the eager kernels (the graph replays of resistance() record no events)
        from fluidlets_gb300.core import _assemble_dev, _mixed_lu_solve_dev

        K = _assemble_dev(k, X, X, e, 1.0, sym_eps=eps, reciprocal=True)
        L.flg_profile_enable(1)
        _mixed_lu_solve_dev(K, U.reshape(-1), 1e-12, 60, 200, lu, required=1e-10)
        del K
        import ctypes

        upd_ms, upd_n = ctypes.c_double(0), ctypes.c_int64(0)
        L.flg_profile_read(_lib.SLOT["lu_update"], ctypes.byref(upd_ms), ctypes.byref(upd_n))
        app_ms, app_n = ctypes.c_double(0), ctypes.c_int64(0)
        L.flg_profile_read(_lib.SLOT["lu_solve"], ctypes.byref(app_ms), ctypes.byref(app_n))
        L.flg_profile_enable(0)
        n = 3 * n_points
        res[f"mixed_{lu}"]["tensor_updates"] = {"ms": upd_ms.value, "launches": upd_n.value,
                                                "tflops": 2.0 / 3.0 * n ** 3 / (upd_ms.value * 1e-3) / 1e12}
        ld32 = (n + 31) // 32 * 32
        res[f"mixed_{lu}"]["preconditioner_apply"] = {
            "ms_per_application": app_ms.value / max(app_n.value, 1), "applications": app_n.value,
            "gbs": 4.0 * n * ld32 / (app_ms.value / max(app_n.value, 1) * 1e-3) / 1e9,
            "bytes": "L and U once: 4 n^2 bytes (FP32) per application"}
    res["cublas_peaks"] = gemm_peaks(dev)
    for lu in ("tf32", "bf16"):
        peak = res["cublas_peaks"][lu]
        res[f"mixed_{lu}"]["tensor_updates"]["frac_of_cublas"] = res[f"mixed_{lu}"]["tensor_updates"]["tflops"] / peak
        res[f"mixed_{lu}"]["preconditioner_apply"]["frac_of_hbm"] = (
            res[f"mixed_{lu}"]["preconditioner_apply"]["gbs"] / hbm_peak_gbs())
    return res


def hbm_peak_gbs():
    """Measured copy bandwidth of the GB300s (generated MEASURED_PEAKS.json), or the
    stated fallback of 6,800 GB/s when the file is absent."""
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0


def gemm_peaks(dev, n=8192, reps=5):
    """Dense tensor-core denominators for the LU updates: cuBLAS (through torch.matmul) TF32 and BF16
    GEMMs of n^3, best of `reps` (CUDA events), in TFLOP/s."""
    import torch

    out = {}
    prev = torch.backends.cuda.matmul.allow_tf32
    try:
        for name, dt in (("tf32", torch.float32), ("bf16", torch.bfloat16)):
            torch.backends.cuda.matmul.allow_tf32 = name == "tf32"
            a = torch.randn(n, n, device=dev, dtype=dt)
            b = torch.randn(n, n, device=dev, dtype=dt)
            torch.matmul(a, b)
            best = float("inf")
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                torch.matmul(a, b)
                e1.record()
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1))
            out[name] = 2.0 * n ** 3 / (best * 1e-3) / 1e12
            del a, b
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    out["source"] = f"cuBLAS via torch.matmul, {n}^3, best of {reps} (measured in this run)"
    return out


def serve_section(n_requests=512, rate=200.0, slots=6):
    """A short served run of the mixed workload (the serve workload's generator): n_requests
    Poisson arrivals at `rate`/s through the continuous-batching server; p50 / p99 latency and
    solves/s (warm-up and per-bucket autotuning before the timed run)."""
    from fluidlets_gb300.serve import serve_run

    return serve_run(n_requests=n_requests, rate=rate, slots=slots)


def run_ours(args):
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import fluidlets_gb300 as fl
    from fluidlets_gb300 import _lib

    L = _lib.load()
    dev = torch.device("cuda", local)
    T, S, F, eps = make_workload(rank)
    Td, Sd, Fd = (torch.from_numpy(a).to(dev) for a in (T, S, F))
    ed = torch.full((N_SRC,), eps, dtype=torch.float64, device=dev)
    kern = fl.WallStokeslet3D()
    pairs = len(T) * len(S)
    flush = torch.empty(256 * 2**20, dtype=torch.uint8, device=dev)

    import ctypes

    fp32_peak, fp64_peak = ctypes.c_double(0), ctypes.c_double(0)
    _lib.check(L.flg_measure_peaks(ctypes.byref(fp32_peak), ctypes.byref(fp64_peak),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))

    def step():
        return fl.evaluate(kern, Td, Sd, Fd, ed, precision="mixed")

    for _ in range(args.warmup):
        out = step()
    torch.cuda.synchronize()
    L.flg_profile_enable(1)
    launches0 = L.flg_launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            ev[k][0].record()
            out = step()
            ev[k][1].record()
            flush.zero_()  # L2 flush between timed steps (outside the event pair)
        torch.cuda.synchronize()
    launches = L.flg_launch_count() - launches0
    if dist:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    far_ms, far_n = ctypes.c_double(0), ctypes.c_int64(0)
    L.flg_profile_read(_lib.SLOT["far_f32"], ctypes.byref(far_ms), ctypes.byref(far_n))
    near_ms, near_n = ctypes.c_double(0), ctypes.c_int64(0)
    L.flg_profile_read(_lib.SLOT["near_f64"], ctypes.byref(near_ms), ctypes.byref(near_n))
    L.flg_profile_enable(0)
    value, total_ms = ranks_throughput(dist, total_ms, pairs * args.steps, world, dev)

    # e2e through the public API: pinned host inputs, host output
    Th, Sh, Fh = (torch.from_numpy(a).pin_memory() for a in (T, S, F))
    out_h = None
    for _ in range(1):
        out_h = fl.evaluate(kern, Th, Sh, Fh, eps, precision="mixed")
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        out_h = fl.evaluate(kern, Th, Sh, Fh, eps, precision="mixed")
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    assert out_h.device.type == "cpu"
    h2d = (T.nbytes + S.nbytes + F.nbytes)
    d2h = out_h.numel() * out_h.element_size()
    e2e_value, _ = ranks_throughput(dist, e2e_s * 1e3, pairs, world, dev, reduce="min")

    far_avg_ms = far_ms.value / max(far_n.value, 1)
    achieved = FLOPS_PER_PAIR * pairs / (far_avg_ms * 1e-3) / 1e12
    traffic, prof_data = None, {}
    prof = ROOT / "profiles" / "far_f32_wall_traffic.json"
    if prof.exists():
        try:
            prof_data = json.loads(prof.read_text())
            traffic = prof_data.get("bytes_per_launch_full_size")
        except (ValueError, OSError):
            traffic = None
    # executed-instruction view beside the canonical-flop fraction: the live pair rate times the
    # instructions per pair that ncu counted, against the issue peak (one warp instruction per
    # SM sub-partition per clock) at the SM clock seen during the timed region
    clocks = clk.summary()
    executed = None
    ipp = prof_data.get("thread_instructions_per_pair")
    if ipp and clocks.get("sm_mhz"):
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        issue_peak = sms * 4 * clocks["sm_mhz"] * 1e6          # warp instructions / s
        achieved_issue = pairs / (far_avg_ms * 1e-3) * ipp / 32  # warp instructions / s
        executed = {"thread_instructions_per_pair": ipp, "issue_frac": achieved_issue / issue_peak,
                    "fma_pipe_pct_ncu": prof_data.get("fma_pipe_pct"),
                    "issue_active_pct_ncu": prof_data.get("issue_active_pct"),
                    "note": "frac above counts canonical flops (106 per pair); the kernel issues fewer "
                            "instructions than that count implies, so its frac can exceed 1 while the "
                            "issue slots are not all used"}
        lane_ops = prof_data.get("fma_lane_ops_per_pair")
        if lane_ops:
            # the FP32 pipe's lane rate (128 per SM per clock, packed FP32x2 or not)
            executed["fma_lane_ops_per_pair"] = lane_ops
            executed["fma_lane_frac"] = pairs / (far_avg_ms * 1e-3) * lane_ops / (sms * 128 * clocks["sm_mhz"] * 1e6)
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 far field + f64 near field (r<4eps)",
        "data": "synthetic (seeded uniform points, N(0,1) forces)",
        "config": {"workload": WORKLOAD, "targets": len(T), "sources": len(S), "eps": eps,
                   "precision": "mixed", "l2": "flushed (256 MB write) between timed steps",
                   "parallelism": f"replicas x{world}"},
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak.value, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak.value, "traffic": traffic,
                     "kernel": "far_f32_kernel", "flops_per_pair": FLOPS_PER_PAIR,
                     "peak_source": "FFMA microbenchmark measured in this run (of measured)",
                     "far_ms_per_launch": far_avg_ms, "near_ms_per_launch": near_ms.value / max(near_n.value, 1),
                     "executed": executed},
        "fp64_peak_tflops": fp64_peak.value,
    }
    if rank == 0 and not args.no_extras:
        # accuracy vs the plain FP64 GPU path on a sample of targets, and that path's rate
        idx = np.r_[np.arange(0, N_TGT, 32), N_TGT + np.arange(0, N_WALL, 16)]
        Ts = Td[torch.from_numpy(idx).to(dev)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u64 = fl.evaluate(kern, Ts, Sd, Fd, ed, precision="fp64")
        torch.cuda.synchronize()
        fp64_rate = len(idx) * N_SRC / (time.perf_counter() - t0)
        um = out[torch.from_numpy(idx).to(dev)]
        inter = torch.from_numpy(idx < N_TGT).to(dev)
        err = float(torch.linalg.vector_norm(um[inter] - u64[inter]) / torch.linalg.vector_norm(u64[inter]))
        line["accuracy"] = {"rel_l2_vs_fp64_gpu": err, "max_abs_u_on_wall_mixed": float(um[~inter].abs().max()),
                            "max_abs_u_on_wall_fp64": float(u64[~inter].abs().max()),
                            "sample_targets": int(len(idx))}
        line["fp64_gpu_path"] = {"value": fp64_rate, "unit": "pairs/s",
                                 "sample": f"{len(idx)} targets x {N_SRC} sources",
                                 "mixed_speedup": value / world / fp64_rate}
        line["solves"] = solve_section(dev)
        line["wall_lu"] = wall_lu_section(dev)
        line["served"] = serve_section()
        sub = cpu_slice(T, args.cpu_sample)
        rate, threads = cpu_sample_rate(sub, S, F, eps)
        line["cpu_baseline"] = {"value": rate, "unit": "pairs/s", "cores": threads, "kind": "port",
                                "sample": f"{len(sub)}-target slice (every {max(1, len(T) // args.cpu_sample)}th "
                                          f"target) x {N_SRC} sources (WallStokeslet3D, FP64); pairs/s scale "
                                          "linearly to the full sum"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_brinkman_gmres(args):
    """Sphere radius 1, N Fibonacci points (default 65,536), eps = 0.2 x mean NN spacing, Brinkmanlet
    alpha in {0, 1, 10} and alpha = (1 + i) sqrt(omega / 2), omega in {1, 10}; rigid translation
    (1, 0, 0) and rotation (0, 0, 1) x x; GMRES(restart 50) to 1e-10: FP32-far/FP64-near matvecs in
    FP64 iterative refinement, and (with --fp64) the plain FP64-matvec GMRES."""
    import torch

    import fluidlets_gb300 as fl
    from fluidlets_gb300.geometry import fibonacci_sphere, mean_nn_spacing

    n = args.n_points or 65536
    X = fibonacci_sphere(n)
    eps = 0.2 * mean_nn_spacing(X)
    dev = torch.device("cuda")
    Xd = torch.from_numpy(X).to(dev)
    ed = torch.full((n,), eps, dtype=torch.float64, device=dev)
    Ut = torch.zeros_like(Xd)
    Ut[:, 0] = 1.0
    Ur = torch.stack([-Xd[:, 1], Xd[:, 0], torch.zeros_like(Xd[:, 0])], 1)  # (0, 0, 1) x x
    out = {"workload": f"Brinkmanlet GMRES, unit sphere N={n} Fibonacci, eps={eps:.7f} (0.2 x mean NN spacing), "
                       "restart 50, rtol 1e-10", "cases": []}
    alphas = [0.0, 1.0, 10.0, (1 + 1j) * np.sqrt(0.5), (1 + 1j) * np.sqrt(5.0)]
    # warm-up (module loading, kernel attributes) outside the timed solves
    fl.resistance(fl.Brinkmanlet3D(1.0), Xd[:512], Ut[:512], ed[:512], method="gmres", precision="mixed")
    for a in alphas:
        k = fl.Brinkmanlet3D(a)
        for motion, U in (("translate_x", Ut), ("rotate_z", Ur)):
            case = {"alpha": str(a), "motion": motion}
            for prec in (["mixed", "fp64"] if args.fp64 else ["mixed"]):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                F, info = fl.resistance(k, Xd, U, ed, method="gmres", restart=50, maxiter=200, precision=prec)
                torch.cuda.synchronize()
                dt = time.perf_counter() - t0
                Fh = F.cpu().numpy()
                drag = Fh[:, 0].sum()
                torque = (X[:, 0] * Fh[:, 1] - X[:, 1] * Fh[:, 0]).sum()
                case[prec] = {"seconds": dt, "iterations": info.iterations, "ir_steps": info.ir_steps,
                              "residual": info.residual,
                              "drag_x": complex(drag).real if np.iscomplexobj(drag) else float(drag),
                              "torque_z": complex(torque).real if np.iscomplexobj(torque) else float(torque),
                              "drag_x_imag": float(np.imag(drag)), "torque_z_imag": float(np.imag(torque))}
                case[prec + "_forces"] = Fh
            if args.fp64:
                # accuracy against the FP64 solution converged to 1e-13 (the rtol = 1e-10 FP64 solve
                # above is itself only accurate to ~ condition number x 1e-10)
                Fc, ic = fl.resistance(k, Xd, U, ed, method="gmres", restart=50, maxiter=400, rtol=1e-13)
                Fc = Fc.cpu().numpy()
                for prec in ("mixed", "fp64"):
                    case[f"rel_force_err_{prec}_vs_converged_fp64"] = float(
                        np.linalg.norm(case[prec + "_forces"] - Fc) / np.linalg.norm(Fc))
                case["speedup_mixed_vs_fp64"] = case["fp64"]["seconds"] / case["mixed"]["seconds"]
            for key in [c for c in case if c.endswith("_forces")]:
                del case[key]
            out["cases"].append(case)
            print(json.dumps(case), flush=True)
    print(json.dumps(out), flush=True)


def run_wall_lu(args):
    """Sphere radius 1, N Fibonacci points (default 8,192), centre heights h/a in {1.05, 1.5, 3.0}
    over the wall z = 0, eps = 0.25 x mean NN spacing, WallStokeslet3D, translation parallel (x)
    and normal (z): TF32 and BF16 tensor-core LU + FP64 GMRES-IR to 1e-10, against the FP64 LU."""
    import torch

    import fluidlets_gb300 as fl
    from fluidlets_gb300.geometry import fibonacci_sphere, mean_nn_spacing

    n = args.n_points or 8192
    S = fibonacci_sphere(n)
    eps = 0.25 * mean_nn_spacing(S)
    dev = torch.device("cuda")
    ed = torch.full((n,), eps, dtype=torch.float64, device=dev)
    k = fl.WallStokeslet3D()
    out = {"workload": f"WallStokeslet3D dense LU, sphere N={n} ({3 * n} unknowns), eps={eps:.7f}", "cases": []}
    for h in (1.05, 1.5, 3.0):
        Xd = torch.from_numpy(S + [0, 0, h]).to(dev)
        for motion, vec in (("parallel_x", [1.0, 0, 0]), ("normal_z", [0, 0, 1.0])):
            U = torch.tensor(vec, dtype=torch.float64, device=dev).expand(n, 3).contiguous()
            case = {"h_over_a": h, "motion": motion}
            ref = None
            if args.fp64:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                F64, i64 = fl.resistance(k, Xd, U, ed, method="lu")
                torch.cuda.synchronize()
                case["fp64_lu"] = {"seconds": time.perf_counter() - t0, "residual": i64.residual,
                                   "drag": float(F64[:, 0 if motion == "parallel_x" else 2].sum())}
                ref = F64
            for lu in ("tf32", "bf16"):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                Fm, im = fl.resistance(k, Xd, U, ed, method="lu", precision="mixed", lu=lu)
                torch.cuda.synchronize()
                c = {"seconds": time.perf_counter() - t0, "residual": im.residual, "ir_steps": im.ir_steps,
                     "gmres_iterations": im.iterations,
                     "drag": float(Fm[:, 0 if motion == "parallel_x" else 2].sum())}
                if ref is not None:
                    c["rel_force_err_vs_fp64"] = float(torch.linalg.vector_norm(Fm - ref) / torch.linalg.vector_norm(ref))
                    c["speedup_vs_fp64"] = case["fp64_lu"]["seconds"] / c["seconds"]
                case["mixed_" + lu] = c
            out["cases"].append(case)
            print(json.dumps(case), flush=True)
    print(json.dumps(out), flush=True)


def run_case(a):
    """One hot-path operation at a chosen size (for profiler captures); inputs are the seeded
    synthetic workloads of this file at reduced size."""
    import torch

    import fluidlets_gb300 as fl
    from fluidlets_gb300 import core
    from fluidlets_gb300.geometry import fibonacci_sphere, mean_nn_spacing, wall_sum_workload

    dev = torch.device("cuda")
    kern = {"stokeslet": fl.Stokeslet3D(), "wall": fl.WallStokeslet3D()}.get(a.kind) or fl.Brinkmanlet3D(a.alpha)
    if a.case == "sum":
        T, S, F, eps = wall_sum_workload(a.sources, a.targets, 0, 0.01, seed=0)
        Td, Sd, Fd = (torch.from_numpy(x).to(dev) for x in (T, S, F))
        for _ in range(a.reps):
            fl.evaluate(kern, Td, Sd, Fd, eps, precision=a.precision)
        torch.cuda.synchronize()
    elif a.case == "breakdown":
        case_breakdown(a, kern)
    elif a.case == "lu_batch":
        case_lu_batch(a, kern)
    elif a.case == "swim":
        case_swim(a)
    else:
        X = fibonacci_sphere(a.n) + (np.array([0, 0, 1.5]) if a.kind == "wall" else 0)
        eps = 0.25 * mean_nn_spacing(X)
        Xd = torch.from_numpy(X).to(dev)
        U = torch.zeros_like(Xd)
        U[:, 0] = 1.0
        for _ in range(a.reps):
            t0 = time.perf_counter()
            if a.case == "assemble":
                fl.assemble(kern, Xd, Xd, eps)
            elif a.case == "lu":
                core.resistance(kern, Xd, U, eps, method="lu", precision=a.precision, lu=a.lu)
            else:
                core.resistance(kern, Xd, U, eps, precision=a.precision, lu=a.lu)
            torch.cuda.synchronize()
            print(f"{a.case} n={a.n}: {1e3 * (time.perf_counter() - t0):.2f} ms")


def case_lu_batch(a, kern):
    """A group of nbat resistance systems of one bucket (a.n points each, Fibonacci spheres of
    slightly different radii): one replay of the batched bucket graph (assembly, FP32 copies,
    batched tensor-core LU) against nbat replays of the single-system graph, one after another
    on one stream and side by side on nbat streams; CUDA-event times per group."""
    import ctypes

    import torch

    from fluidlets_gb300 import _device as dv
    from fluidlets_gb300 import _lib
    from fluidlets_gb300.geometry import fibonacci_sphere, mean_nn_spacing

    L = _lib.load()
    dev = torch.device("cuda")
    code, nbat, n_cap = _lib.KIND[a.kind], a.nbat, a.n
    n, ld32 = 3 * n_cap, (3 * n_cap + 31) // 32 * 32
    mode = _lib.lu_mode(a.lu)
    pts = np.stack([fibonacci_sphere(n_cap) * (1.0 + 0.05 * z) + ([0, 0, 1.5] if a.kind == "wall" else 0)
                    for z in range(nbat)])
    eps = np.stack([np.full(n_cap, 0.25 * mean_nn_spacing(pts[z])) for z in range(nbat)])
    P, E = torch.tensor(pts, device=dev), torch.tensor(eps, device=dev)
    NR = torch.full((nbat,), n_cap, dtype=torch.int64, device=dev)
    bufs = dict(K=torch.empty((nbat, n, n), dtype=torch.float64, device=dev),
                K32=torch.empty((nbat, n, ld32), dtype=torch.float32, device=dev),
                A32=torch.empty((nbat, n, ld32), dtype=torch.float32, device=dev),
                dinv=torch.empty((nbat, L.flg_lu_lowp_dinv_elems(n)), dtype=torch.float32, device=dev),
                flags=torch.zeros(2 * nbat, dtype=torch.int32, device=dev))
    streams = [torch.cuda.Stream() for _ in range(nbat)]
    sp = [ctypes.c_void_p(s.cuda_stream) for s in streams]

    def graph(z0, k, st):
        wb = L.flg_lu_factor_lowp_batched_workspace(n, k, mode) if k > 1 else L.flg_lu_factor_lowp_workspace(n, mode)
        ws = dv.workspace(wb)
        h = ctypes.c_void_p(0)
        args = (code, 0.0, 0.0, dv.ptr(P[z0]), dv.ptr(E[z0]), 1, dv.ptr(NR[z0:]), n_cap)
        tail = (1.0, dv.ptr(bufs["K"][z0]), dv.ptr(bufs["A32"][z0]), dv.ptr(bufs["K32"][z0]), ld32, mode,
                dv.ptr(bufs["dinv"][z0]), dv.ptr(bufs["flags"][2 * z0:]), dv.ptr(ws), wb, st, ctypes.byref(h))
        _lib.check(L.flg_bucket_batch_graph_create(*args, k, *tail) if k > 1 else
                   L.flg_bucket_graph_create(*args, *tail), "graph")
        return h, ws

    gb = graph(0, nbat, sp[0])
    gs = [graph(z, 1, sp[z]) for z in range(nbat)]
    torch.cuda.synchronize()

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms = []
        for _ in range(max(a.reps, 3)):
            e0.record(streams[0])
            fn()
            for s in streams[1:]:  # the other streams' work joins stream 0 before the end event
                ev = torch.cuda.Event()
                ev.record(s)
                streams[0].wait_event(ev)
            e1.record(streams[0])
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return min(ms)

    def batched():
        L.flg_graph_launch(gb[0], sp[0])

    def sequential():
        for z in range(nbat):
            L.flg_graph_launch(gs[z][0], sp[0])

    def side_by_side():
        ev = torch.cuda.Event()
        ev.record(streams[0])
        for z in range(nbat):
            streams[z].wait_event(ev)
            L.flg_graph_launch(gs[z][0], sp[z])

    tb, tq, tp = timed(batched), timed(sequential), timed(side_by_side)
    assert not bufs["flags"].any()
    print(f"[lu_batch {a.kind} {a.lu}] {nbat} systems of n = {n}: batched graph {tb:.3f} ms, "
          f"{nbat} single graphs in turn {tq:.3f} ms, side by side on {nbat} streams {tp:.3f} ms")
    for h, _ in [gb] + gs:
        L.flg_graph_destroy(h)


def case_swim(a):
    """swim() of the biflagellate swimmer over one beat period (RK45, rtol 1e-6): FP64 solves per
    stage vs the captured mixed-precision stage graph; time per right-hand side.  Flagellum
    amplitude 0.08, so the two mirror-image flagella (attached at z = +-0.1) never touch (with 0.2
    they cross and the system is near-singular there); nearest map fixed at t = 0 (the flagellum
    quadrature points sit midway between force points, so a recomputed map would flip and make
    the right-hand side discontinuous)."""
    import torch

    import fluidlets_gb300 as fl
    from fluidlets_gb300.geometry import biflagellate_shape

    calls = {"n": 0}

    def shape_at(t):
        calls["n"] += 1
        return biflagellate_shape(t, amplitude=0.08)

    s0 = biflagellate_shape(0.0, amplitude=0.08)
    out = {}
    for prec in ("fp64", "mixed", "mixed"):  # the second mixed run is timed warm
        calls["n"] = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tr = fl.swim(shape_at, (0.0, 1.0), 0.02, rtol=1e-6, atol=1e-9, fixed_nearest=True, precision=prec)
        torch.cuda.synchronize()
        out[prec] = (time.perf_counter() - t0, calls["n"], tr)
    t64, n64, tr64 = out["fp64"]
    tmx, nmx, trmx = out["mixed"]
    dx = np.abs(tr64.x0[-1] - trmx.x0[-1]).max()
    print(f"swim: N={len(s0.x)} force / {len(s0.X)} quadrature points, n={3 * len(s0.x) + 6}; "
          f"fp64 {t64 * 1e3:.0f} ms for {n64} right-hand sides ({t64 / n64 * 1e3:.2f} ms each); "
          f"mixed {tmx * 1e3:.0f} ms for {nmx} ({tmx / nmx * 1e3:.2f} ms each); final position difference {dx:.1e}")


def case_breakdown(a, kern):
    """Phase times of one mixed-precision dense resistance solve (assembly, FP32 copy,
    tensor-core LU, FP64 GMRES-IR, final FP64 residual) and of the FP64 LU."""
    import ctypes

    import torch

    from fluidlets_gb300 import _lib, core
    from fluidlets_gb300.geometry import fibonacci_sphere, mean_nn_spacing

    L = _lib.load()
    dev = torch.device("cuda")
    X = fibonacci_sphere(a.n) + (np.array([0, 0, 1.5]) if a.kind == "wall" else 0)
    eps = 0.25 * mean_nn_spacing(X)
    Xd = torch.from_numpy(X).to(dev)
    e = torch.full((a.n,), eps, dtype=torch.float64, device=dev)
    U = torch.zeros_like(Xd)
    U[:, 0] = 1.0
    b = U.reshape(-1).contiguous()

    def t(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, 1e3 * (time.perf_counter() - t0)

    for rep in range(a.reps):
        L.flg_profile_enable(1)
        K, t_asm = t(lambda: core._assemble_dev(kern, Xd, Xd, e, 1.0, sym_eps=eps, reciprocal=True))
        (K32, ld32, dinv, A32), t_lu = t(lambda: core._lowp_factor_dev(K, a.lu))
        (x, it, outer, res), t_ir = t(lambda: core._gmres_ir_dense_dev(K, K32, ld32, dinv, b, 1e-12, 60, 200,
                                                                        required=1e-10, A32=A32))
        _, t_res = t(lambda: core._evaluate_dev(kern, Xd, Xd, x.reshape(-1, 3), e, 1.0, "fp64"))
        slots = {}
        for name, k in _lib.SLOT.items():
            ms, n = ctypes.c_double(0), ctypes.c_int64(0)
            L.flg_profile_read(k, ctypes.byref(ms), ctypes.byref(n))
            if n.value:
                slots[name] = (round(ms.value, 3), n.value)
        L.flg_profile_enable(0)
        print(f"[mixed {a.lu}] n={3 * a.n}: assemble {t_asm:.2f} ms, convert+LU {t_lu:.2f} ms, GMRES-IR {t_ir:.2f} ms "
              f"({it} it, {outer} IR, resid {res:.2e}), residual {t_res:.2f} ms; kernel slots (ms, launches): {slots}")
    if a.n > 4096:  # the FP64 factorizations take seconds at this size
        return
    K = core._assemble_dev(kern, Xd, Xd, e, 1.0)
    L.flg_profile_enable(1)
    _, t64 = t(lambda: core._lu_solve_dev(K.clone(), b))
    slots = {}
    for name, k in _lib.SLOT.items():
        ms, n = ctypes.c_double(0), ctypes.c_int64(0)
        L.flg_profile_read(k, ctypes.byref(ms), ctypes.byref(n))
        if n.value:
            slots[name] = (round(ms.value, 3), n.value)
    L.flg_profile_enable(0)
    print(f"[fp64] kernel slots (ms, launches): {slots}")
    torch.linalg.solve(K, b)  # library initialization outside the timing
    _, tcs = t(lambda: torch.linalg.solve(K, b))
    print(f"[fp64] LU factor+solve {t64:.2f} ms; cuSOLVER (torch.linalg.solve) {tcs:.2f} ms")



def main():
    args = parse()
    if args.case:
        return run_case(args)
    if args.impl != "reference" and args.workload == "brinkman_gmres":
        return run_brinkman_gmres(args)
    if args.impl != "reference" and args.workload == "wall_lu":
        return run_wall_lu(args)
    if args.impl != "reference" and args.workload == "serve":
        from fluidlets_gb300.serve import bench_serving
        return bench_serving(args)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
