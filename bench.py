"""Benchmark: RK4 steps/s of the Roberts-1983 boundary-integral step on GB300.

Workload (the headline configuration): gravity wave, N = 4096 nodes, 8 seeded
modes (a_m ~ U(0,0.02)/m, theta_m ~ U(0,2 pi), seed 2), phi from the linear
dispersion relation, g = 1, RK4 dt = 0.005, mixed precision (FP32
preconditioner + double-float / FP64 refinement).  Synthetic data: the
reference measures on no dataset.

The one JSON line carries:
  value  : mixed-precision steps/s with the state resident in HBM: one CUDA
           event pair on the engine stream around the K steps and the L2 flush
           (a 256 MB write) before each, minus K flushes timed alone; the
           background preconditioner rebuild (refactor_lag) is joined before
           the end event
  e2e    : steps/s through the C ABI with host buffers (pinned host -> device
           copy of the state, one step, device -> host copy, every step)
  fp64   : the plain FP64 GPU step (the engine in FP64 mode: assembled FP64
           matrix, blocked FP64 LU, FP64 sums) on the same surface, event-timed;
           mixed_over_fp64 = value / its steps/s (the metric's ratio)
  accuracy: max|z_mixed - z_fp64| / max|z_fp64| and the same for phi after 25,
           50 and 100 steps (the benchmarked mixed settings), beside the FP64
           round-off envelope: the FP64 run against an FP64 run whose x was
           perturbed by 1e-15 relative
  roofline: the dominant kernel class of the step (largest device time per
           step in an event-timed pass, graphs off) against the measured peak
           of the unit that bounds it; every class with its algorithmic work,
           achieved rate and fraction in roofline.classes.  Peaks: HBM and
           bf16 from MEASURED_PEAKS.json, FP64 and FP32 (SIMT) from cuBLAS
           DGEMM / SGEMM (TF32 off) timed here before the timed region
  cpu_baseline: the FP64 CPU oracle (a port of the reference path, OpenMP over
           the host's cores), median of 3 RK4 steps at N = 4096
  adjoint: the hand-written adjoint on the fit workload, on a mixed engine
           against its own recorded forward (the headline ratio) and on an
           FP64 engine likewise, with the two gradients compared
  helium_batch: 512 uneven helium films in one mixed engine (surface-steps/s,
           error against the FP64 engine after 5 steps, per-surface status)

--impl reference runs the reference-side CPU path (the oracle port: the
reference's CUDA path does not compile from its sources as they lie and its
NumPy calculator cannot be shipped) on the same workload and prints the same
line with "impl": "reference"; under torchrun rank 0 alone runs it.

Our arm under torchrun (N > 1) runs an independent replica per rank (a single
surface does not shard); value = all ranks' steps / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK4 steps/s at N=4096, mixed vs FP64 GPU at ≤1e-9 rel error; adjoint/fwd ratio"
N_NODES = 4096
DT = 0.005


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), float(d.get("bf16_tflops_sustained", d["bf16_tflops"])), "measured"
    except Exception:
        return 6800.0, 1900.0, 1700.0, "fallback"


def simt_peaks(device: int) -> dict:
    """FP64 and FP32 (SIMT) peaks of this GPU, measured as cuBLAS DGEMM and
    SGEMM with TF32 off (best of 5 after 3 warm-ups, CUDA events): the
    denominators of the FP64- and FP32-bound kernel classes."""
    import torch
    dev = torch.device("cuda", device)
    out = {}
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        for name, dtype, n in (("fp64_tflops", torch.float64, 4096), ("fp32_tflops", torch.float32, 8192)):
            a = torch.randn(n, n, device=dev, dtype=dtype)
            b = torch.randn(n, n, device=dev, dtype=dtype)
            for _ in range(3):
                torch.matmul(a, b)
            best = float("inf")
            for _ in range(5):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                torch.matmul(a, b)
                e1.record()
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1) * 1e-3)
            out[name] = 2.0 * n ** 3 / best / 1e12
            del a, b
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    torch.cuda.empty_cache()
    out["method"] = "cuBLAS DGEMM n=4096 / SGEMM n=8192 (TF32 off), best of 5, CUDA events"
    return out


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                p = [v.strip() for v in line.split(",")]
                if len(p) >= 9 and p[1].replace(".", "").isdigit():
                    rows.append(p)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows]
        mx = float(rows[0][2])
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(rows)}


def kernel_traffic(kernel: str, n: int):
    """DRAM bytes (read + write) per launch of `kernel` at N = n from the
    committed ncu summaries under profiles/ (a line
    `dram_bytes_per_launch kernel=<name> n=<N>: <bytes>`), or None."""
    key = f"dram_bytes_per_launch kernel={kernel} n={n}:"
    d = os.path.join(ROOT, "profiles")
    try:
        names = sorted(os.listdir(d))
    except OSError:
        return None
    for name in names:
        try:
            with open(os.path.join(d, name)) as f:
                for line in f:
                    line = line.strip().strip("`")
                    if line.startswith(key):
                        return float(line[len(key):].split()[0])
        except OSError:
            continue
    return None


# Algorithmic work of the kernel classes, per unit, as the roofline counts it.
#   spectral_deriv     : per transform job (forward + inverse complex FFT of n
#                        points, 5 n log2 n FLOP each): 10 n log2 n FP64 FLOP
#   boundary_sums_fp32 : per (target, source) pair, water: 15 FP32 FLOP (two
#                        double-float-split differences, |d|^2, reciprocal
#                        estimate, weight, two FMA accumulations)
#   boundary_sums_df   : per pair, water: 77 FP32 FLOP, FMA = 2 (double-float
#                        difference renormalised by a quick two-sum, squared
#                        norm, quotient with one remainder correction, the two
#                        products with d, cascaded accumulation; packed
#                        FP32x2 lanes count twice)
#   boundary_sums_fp64 : per pair, water: 11 FP64 FLOP
#   gemv               : per product: 2 n^2 bytes (the FP16 preconditioner)
#   fft4_columns, fft4_rows, fft4_inverse_columns (four-step transforms of a
#                        power-of-two n = 64 N2 on the step's critical path;
#                        per RK stage z is transformed forward once and back
#                        twice, phi forward and back once): 5 L log2 L FP64
#                        FLOP per length-L FFT, 2 x 64 forward columns
#                        (L = N2), 5 x N2 rows (L = 64), 3 x 64 inverse
#                        columns per stage
#   ap_transform       : the a' transform of each stage (forked beside the
#                        last boundary-sum pass while stepping on graphs):
#                        four-step, 64 forward columns, 2 x N2 rows, 64
#                        inverse columns; otherwise 10 n log2 n per stage
#   start_product      : a0 = X phi', returning at once on warm starts:
#                        reported by time only
#   node_prep, velocity_bernoulli, rk4_combine: O(n), reported by time only
#   extra_corrections, ap_redo: the gated extra corrections and the a'
#                        transform repeated after them; they return at once
#                        where the residual is converged (no work counted),
#                        reported by time only
FLOP_PER_PAIR = {"boundary_sums_fp32": 15.0, "boundary_sums_df": 77.0, "boundary_sums_fp64": 11.0}


def fft4_work_per_step(cls: str, n: int) -> float:
    """FP64 FLOP per RK4 step of one four-step transform class (n = 64 N2)."""
    n2 = n // 64
    col = 5.0 * n2 * math.log2(n2)
    row = 5.0 * 64 * 6
    return 4 * {"fft4_columns": 2 * 64 * col, "fft4_rows": 5 * n2 * row, "fft4_inverse_columns": 3 * 64 * col,
                "ap_transform": 2 * 64 * col + 2 * n2 * row}[cls]


def class_roofline(prof: dict, prof_steps: int, n: int, sums_per_step: dict, jobs_per_step: int,
                   gemv_per_step: int, pk: dict) -> dict:
    """Per kernel class: ms per step, algorithmic work per step, achieved rate
    and fraction of the bounding unit's measured peak."""
    classes = {}
    for name, (tms, cnt) in prof.items():
        if not cnt:
            continue
        ms = tms / prof_steps
        c = {"ms_per_step": round(ms, 5), "launches_per_step": round(cnt / prof_steps, 3)}
        sec = ms * 1e-3
        if name == "spectral_deriv":
            work = jobs_per_step * 10.0 * n * math.log2(n)
            c.update(bound="fp64", unit="TFLOP/s", work_per_step=work, achieved=work / sec / 1e12,
                     peak=pk["fp64_tflops"])
        elif name.startswith("fft4_") or (name == "ap_transform" and n >= 512 and (n & (n - 1)) == 0):
            work = fft4_work_per_step(name, n)
            c.update(bound="fp64", unit="TFLOP/s", work_per_step=work, achieved=work / sec / 1e12,
                     peak=pk["fp64_tflops"])
        elif name == "ap_transform":
            work = 4 * 10.0 * n * math.log2(n)
            c.update(bound="fp64", unit="TFLOP/s", work_per_step=work, achieved=work / sec / 1e12,
                     peak=pk["fp64_tflops"])
        elif name in FLOP_PER_PAIR:
            passes = sums_per_step.get(name, 0)
            work = passes * float(n) * (n - 1) * FLOP_PER_PAIR[name]
            bound = "fp64" if name.endswith("fp64") else "fp32"
            c.update(bound=bound, unit="TFLOP/s", work_per_step=work, achieved=work / sec / 1e12,
                     peak=pk["fp64_tflops"] if bound == "fp64" else pk["fp32_tflops"])
        elif name == "gemv":
            work = gemv_per_step * 2.0 * n * n
            c.update(bound="hbm", unit="GB/s", work_per_step=work, achieved=work / sec / 1e9, peak=pk["hbm_gbs"])
        if "achieved" in c:
            c["frac"] = c["achieved"] / c["peak"]
        classes[name] = c
    return classes


def adjoint_ratio(device: int, steps: int = 500, every: int = 50):
    """Cost of the hand-written adjoint against the forward pass on the fit
    workload: helium film N=512, h0=10, A3=1e3, 500 RK4 steps at dt=1e-3,
    initial y from 64 seeded Fourier coefficients, checkpoints every 50 steps,
    loss = 0.5 |y_final - y_target|^2.  Wall-clock, synchronous.
      mixed (the headline): forward = sfd_rk4_record on a mixed engine (its
        captured step graphs, preconditioner rebuilt every 50 steps) keeping
        the checkpoints; adjoint = sfd_rk4_vjp (each segment recomputed on the
        mixed engine with every stage recorded, then reversed with the
        X^T-preconditioned transposed solve);
      fp64: the same on an FP64 engine (LU factors recorded per stage).
    The gradients of the two are compared (relative to the FP64 one's largest
    entry)."""
    import superfluid_dynamics_gb300 as sfd
    from superfluid_dynamics_gb300 import workloads
    n, dt = 512, 1e-3
    s, c0, target = workloads.helium_fit(n)
    state0 = np.concatenate([s.x, s.y, s.phi])
    phys = sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3)
    out = {"workload": f"helium film N=512, h0=10, A3=1e3, {steps} RK4 steps dt=1e-3, 64 Fourier coefficients, "
                       f"checkpoints every {every}"}
    grads = {}
    for name, opts in (("mixed", sfd.Options(precision=sfd.PRECISION_MIXED, refactor_every=50, pre_iters=2,
                                             autotune=False, device=device)),
                       ("fp64", sfd.Options(precision=sfd.PRECISION_FP64, use_graphs=False, device=device))):
        eng = sfd.Engine(n, phys, opts)
        # warm-up: workspace and first launches; on the mixed engine the whole
        # workload once, which captures its step graphs (one per step slot of
        # a segment, reused by every later call)
        eng.rk4_record(dt, steps if name == "mixed" else 5, every, state0)
        eng.rk4_vjp(np.zeros(3 * n))
        t0 = time.perf_counter()
        final = eng.rk4_record(dt, steps, every, state0)
        t_fwd = time.perf_counter() - t0
        cot = np.zeros(3 * n)
        cot[n:2 * n] = final[n:2 * n] - target
        eng.clear_status()
        t0 = time.perf_counter()
        g, gp = eng.rk4_vjp(cot)
        t_adj = time.perf_counter() - t0
        st = int(eng.status()[0][0])
        res, corr = eng.adjoint_residual()
        eng.close()
        grads[name] = (g, gp)
        out[name] = {"forward_s": t_fwd, "adjoint_s": t_adj, "ratio": t_adj / t_fwd, "status": st,
                     "loss": 0.5 * float(cot[n:2 * n] @ cot[n:2 * n]), "grad_A3": gp}
        if name == "mixed":
            out[name]["transposed_solve_max_rel_residual"] = res
            out[name]["transposed_solve_max_corrections"] = corr
    out["forward_s"] = out["mixed"]["forward_s"]
    out["adjoint_s"] = out["mixed"]["adjoint_s"]
    out["ratio"] = out["mixed"]["ratio"]
    gm, g64 = grads["mixed"][0], grads["fp64"][0]
    out["mixed_vs_fp64_grad_rel"] = float(np.abs(gm - g64).max() / np.abs(g64).max())
    out["mixed_vs_fp64_grad_A3_rel"] = abs(grads["mixed"][1] - grads["fp64"][1]) / abs(grads["fp64"][1])
    return out


def cpu_sample(steps: int = 1, n: int = N_NODES):
    """Oracle port (FP64, OpenMP over all host cores): time `steps` RK4 steps
    one by one; returns (steps/s from the median step, cores, per-step s)."""
    from oracle import oracle
    from superfluid_dynamics_gb300 import workloads
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    s = workloads.random_modes(n, seed=2)
    x, y, phi = s.x, s.y, s.phi
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        (x, y, phi), _ = oracle.rk4_steps(oracle.Problem(), x, y, phi, DT, 1)
        times.append(time.perf_counter() - t0)
    return 1.0 / statistics.median(times), cores, times


def run_reference(args, rank, world):
    if rank != 0:
        return
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 2))
    if warm:
        cpu_sample(warm)
    rate, cores, _ = cpu_sample(steps)
    line = {"metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": world, "steps": steps, "warmup": warm,
            "ms_per_step": 1e3 / rate, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded 8-mode gravity wave)", "impl": "reference",
            "config": {"workload": f"gravity wave N={N_NODES}, 8 modes seed 2, RK4 dt={DT}", "N": N_NODES,
                       "precision": "fp64", "path": "CPU FP64 oracle port of the reference RHS + RK4"},
            "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": f"median of {steps} RK4 step(s) at N={N_NODES} (of the requested {args.steps})"},
            "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _timed_steps(eng, dt, steps, stream):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
        eng.step(dt, steps, sync=False)
        e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) * 1e-3


def fp64_and_accuracy(args, opts_mixed, device, stream, checkpoints=(25, 50, 100)):
    """The plain FP64 GPU step on the headline surface (event-timed over the
    accuracy run) and the mixed-vs-FP64 error at the checkpoints beside the
    FP64 round-off envelope."""
    import superfluid_dynamics_gb300 as sfd
    from superfluid_dynamics_gb300 import workloads
    n = args.n
    s = workloads.random_modes(n, seed=2)
    fp64 = sfd.Options(precision=sfd.PRECISION_FP64, device=device)
    runs = {}
    for name, opt, eps in (("mixed", opts_mixed, 0.0), ("fp64", fp64, 0.0), ("fp64_perturbed", fp64, 1e-15)):
        eng = sfd.Engine(n, sfd.WaterBoundaryProblem(), opt)
        eng.set_stream(stream.cuda_stream)
        x = s.x * (1 + eps * np.random.default_rng(7).standard_normal(n)) if eps else s.x
        eng.set_state(x, s.y, s.phi)
        traj, t, done = [], 0.0, 0
        for c in checkpoints:
            t += _timed_steps(eng, DT, c - done, stream)
            done = c
            traj.append(np.concatenate(eng.get_state()))
        st = eng.status()
        runs[name] = (traj, done / t, st, eng.refinement() if name == "mixed" else None)
        eng.close()
    fp64_rate = runs["fp64"][1]
    return {
        "fp64": {"steps_per_s": fp64_rate, "steps": checkpoints[-1], "ms_per_step": 1e3 / fp64_rate,
                 "path": "engine FP64 mode: FP64 M assembled, blocked FP64 LU (64-wide), FP64 sums, FP64 FFT",
                 "status_or": int(np.bitwise_or.reduce(runs["fp64"][2][0]))},
        "accuracy": {"steps": list(checkpoints),
                     "mixed_vs_fp64_z_phi": [_state_err(a, b, n) for a, b in zip(runs["mixed"][0], runs["fp64"][0])],
                     "fp64_perturbed_vs_fp64_z_phi": [_state_err(a, b, n) for a, b in
                                                      zip(runs["fp64_perturbed"][0], runs["fp64"][0])],
                     "perturbation": "x * (1 + 1e-15 N(0,1)), seed 7",
                     "mixed_status_or": int(np.bitwise_or.reduce(runs["mixed"][2][0])),
                     "mixed_max_rel_residual": float(runs["mixed"][3]["rel_residual"].max()),
                     "mixed_extra_corrections": int(runs["mixed"][3]["extra_iters"].sum()),
                     "mixed_stall_rebuilds": runs["mixed"][3]["stall_rebuilds"]},
    }


def helium_batch_summary(args, device, stream, timed_steps=50):
    """512 uneven helium films (N = 32 U{4..64}, seed 3) in one mixed engine
    with the headline's solver settings (background rebuild included):
    surface-steps/s over `timed_steps` steps after 5 checked ones, error of
    those 5 steps against the FP64 engine, per-surface status counts."""
    import superfluid_dynamics_gb300 as sfd
    from superfluid_dynamics_gb300 import workloads
    surfs = workloads.helium_batch(512, seed=3)
    ns = [sf.n for sf in surfs]
    phys = [sfd.HeliumBoundaryProblem(depth=sf.depth, A3=sf.A3) for sf in surfs]
    x = np.concatenate([sf.x for sf in surfs])
    y = np.concatenate([sf.y for sf in surfs])
    ph = np.concatenate([sf.phi for sf in surfs])
    dt = 1e-3
    opt = sfd.Options(precision=sfd.PRECISION_MIXED, refine_iters=args.refine_iters, pre_iters=args.pre_iters,
                      refactor_every=args.refactor_every, refactor_lag=args.refactor_lag, device=device)
    eng = sfd.Engine(ns, phys, opt)
    eng.set_stream(stream.cuda_stream)
    eng.set_state(x, y, ph)
    _timed_steps(eng, dt, 5, stream)
    m5 = np.concatenate(eng.get_state())
    t = _timed_steps(eng, dt, timed_steps, stream)
    st = eng.status()[0]
    eng.close()
    ref = sfd.Engine(ns, phys, sfd.Options(precision=sfd.PRECISION_FP64, device=device))
    ref.set_state(x, y, ph)
    ref.step(dt, 5)
    f5 = np.concatenate(ref.get_state())
    ref.close()
    nt = sum(ns)
    off = np.concatenate([[0], np.cumsum(ns)])
    errs = []
    for i in range(len(ns)):
        sl = [slice(k * nt + off[i], k * nt + off[i + 1]) for k in range(3)]
        errs.append(_state_err(np.concatenate([m5[q] for q in sl]), np.concatenate([f5[q] for q in sl]), ns[i]))
    errs = np.array(errs)
    return {"workload": "512 helium films, N = 32 U{4..64} (seed 3), h0 ~ U(5,20), A3 ~ U(0.5,2)e3, dt=1e-3",
            "surface_steps_per_s": len(ns) * timed_steps / t, "steps_per_s": timed_steps / t,
            "timed_steps": timed_steps, "total_nodes": int(nt),
            "max_err_vs_fp64_after_5_steps_z_phi": [float(errs[:, 0].max()), float(errs[:, 1].max())],
            "surfaces_nonfinite": int(((st & sfd._lib.STATUS_NONFINITE) != 0).sum()),
            "surfaces_refine_stall": int(((st & sfd._lib.STATUS_REFINE_STALL) != 0).sum()),
            "surfaces_zero_pivot": int(((st & sfd._lib.STATUS_ZERO_PIVOT) != 0).sum())}


def run_ours(args, rank, world, local_rank):
    import torch
    import superfluid_dynamics_gb300 as sfd
    from superfluid_dynamics_gb300 import workloads

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    pk = {}
    if rank == 0 and not args.no_roofline:
        pk = simt_peaks(local_rank)
    s = workloads.random_modes(args.n, seed=2)
    prec = sfd.PRECISION_MIXED if args.precision == "mixed" else sfd.PRECISION_FP64
    opts = sfd.Options(precision=prec, refine_iters=args.refine_iters, refactor_every=args.refactor_every,
                       pre_iters=args.pre_iters, device=local_rank, precond_half=not args.precond_fp32,
                       refactor_lag=args.refactor_lag, extra_iters=args.extra_iters)
    eng = sfd.Engine(args.n, sfd.WaterBoundaryProblem(), opts)
    stream = torch.cuda.Stream(device=dev)
    eng.set_stream(stream.cuda_stream)
    eng.set_state(s.x, s.y, s.phi)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # warm-up (also builds the CUDA graphs), then untimed steps up to the next
    # preconditioner rebuild so that the timed window starts with one and holds
    # ceil(steps / refactor_every) of them
    warm = args.warmup
    every = max(1, args.refactor_every)
    warm += (every - warm % every) % every if args.precision == "mixed" else 0
    for _ in range(warm):
        eng.step(DT, 1)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    # ---- device-resident timed region: one event pair around the K steps and
    # the L2 flushes between them (any background preconditioner rebuild runs
    # beside them and is joined before the end event), minus K isolated flushes
    with torch.cuda.stream(stream):
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(3):
            flush.fill_(1.0)
        f0.record(stream)
        for _ in range(args.steps):
            flush.fill_(1.0)
        f1.record(stream)
        torch.cuda.synchronize()
    flush_ms = f0.elapsed_time(f1)
    launches0 = eng.kernel_launches
    eng.clear_status()
    with ClockSampler(local_rank) as clk:
        with torch.cuda.stream(stream):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                flush.fill_(1.0)
                eng.step(DT, 1, sync=False)
            eng.join_background()
            e1.record(stream)
            torch.cuda.synchronize()
    gpu_launches = eng.kernel_launches - launches0
    timed_refinement = eng.refinement()
    timed_status = int(np.bitwise_or.reduce(eng.status()[0]))
    tuning = eng.tuning()
    ms = e0.elapsed_time(e1) - flush_ms
    if world > 1:
        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * args.steps / (ms * 1e-3)

    done = warm + args.steps

    def align():
        # untimed steps up to the next preconditioner rebuild
        nonlocal done
        extra = (every - done % every) % every if args.precision == "mixed" else 0
        if extra:
            eng.step(DT, extra)
            done += extra

    # ---- end to end through the C ABI with host buffers: every step is one
    # sfd_rk4_steps_host call that copies the state in from pinned host memory,
    # steps, and copies the result back into the same buffers
    # one pinned [x | y | phi] buffer: the state moves in one copy each way
    buf = torch.from_numpy(np.concatenate([s.x, s.y, s.phi])).pin_memory().numpy()
    x, y, p = buf[:s.x.size], buf[s.x.size:2 * s.x.size], buf[2 * s.x.size:]
    align()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.step_host(x, y, p, DT, 1)
    e2e_s = time.perf_counter() - t0
    done += args.steps
    e2e_value = world * args.steps / e2e_s

    # ---- per-kernel classes (events per launch, graphs off) over one
    # preconditioner period (at most 50 steps)
    eng.set_state(s.x, s.y, s.phi)
    align()
    eng.profile(True)
    prof_steps = min(every, 50) if args.precision == "mixed" else 2
    eng.step(DT, prof_steps)
    prof = eng.profile_read()
    eng.profile(False)
    eng.close()

    if rank != 0:
        return
    hbm, bf16, bf16s, peak_kind = peaks()
    n = args.n
    mixed = args.precision == "mixed"
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64+df32 (mixed)" if mixed else "f64",
            "data": "synthetic (seeded 8-mode gravity wave)",
            "config": {"workload": f"gravity wave N={n}, 8 modes seed 2, RK4 dt={DT}", "N": n,
                       "precision": args.precision, "refine_iters": args.refine_iters, "pre_iters": args.pre_iters,
                       "refactor_every": args.refactor_every, "refactor_lag": args.refactor_lag,
                       "extra_iters": opts.extra_iters, "refine_tol": opts.refine_tol,
                       "precond_storage": "fp32" if args.precond_fp32 else "fp16",
                       "sum_groups_per_cta": tuning,
                       "l2": "flushed (256 MB write) before every timed step",
                       "timing": "CUDA events around the K steps and their L2 flushes (background rebuild joined), "
                                 "minus K flushes timed alone",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": 3 * n * 8,
                    "d2h_bytes_per_step": 3 * n * 8},
            "gpu_launches": gpu_launches, "clocks": clk.summary(),
            "timed_region": {"status_or": timed_status,
                             "max_rel_residual": float(timed_refinement["rel_residual"].max()),
                             "extra_corrections": int(timed_refinement["extra_iters"].sum()),
                             "stall_rebuilds": timed_refinement["stall_rebuilds"]}}

    # ---- the metric's denominator and error bound
    if not args.no_accuracy:
        acc = fp64_and_accuracy(args, opts, local_rank, stream)
        line["fp64"] = acc["fp64"]
        line["fp64_steps_per_s"] = acc["fp64"]["steps_per_s"]
        line["mixed_over_fp64"] = value / acc["fp64"]["steps_per_s"]
        line["accuracy"] = acc["accuracy"]

    # ---- roofline of the dominant kernel class, with every class listed
    if pk:
        pk.update({"hbm_gbs": hbm, "bf16_tflops": bf16, "source_hbm_bf16": peak_kind})
        passes = {"boundary_sums_fp32": 4 * (args.pre_iters + args.refine_iters) if mixed else 0,
                  "boundary_sums_df": 4 if mixed else 0, "boundary_sums_fp64": 0 if mixed else 4}
        gemv = 4 * (args.pre_iters + args.refine_iters) if mixed else 0  # a0 = X phi' is its own class
        f4 = n >= 512 and n <= 8192 and (n & (n - 1)) == 0  # four-step transforms instead of per-job ones
        classes = class_roofline(prof, prof_steps, n, passes, 0 if f4 else 12, gemv, pk)
        dom = max(classes, key=lambda k: classes[k]["ms_per_step"])
        d = classes[dom]
        kname = {"spectral_deriv": "k_spectral_cluster", "boundary_sums_fp32": "k_sums_f32",
                 "boundary_sums_df": "k_sums_dfs", "gemv": "k_gemv_h", "fft4_columns": "k_fft4<1>",
                 "fft4_rows": "k_fft4<2>", "fft4_inverse_columns": "k_fft4<3>"}.get(dom, dom)
        per_launch_work = d.get("work_per_step", 0.0) / max(d["launches_per_step"], 1e-9)
        traffic = kernel_traffic(kname, n)
        line["roofline"] = {
            "bound": d.get("bound"), "kernel": kname, "class": dom, "achieved": d.get("achieved"),
            "peak": d.get("peak"), "unit": d.get("unit"), "frac": d.get("frac"),
            "traffic": traffic, "algorithmic_work_per_launch": per_launch_work,
            "avg_launch_ms": d["ms_per_step"] / max(d["launches_per_step"], 1e-9),
            "peak_source": ("measured cuBLAS DGEMM" if d.get("bound") == "fp64" else
                            "measured cuBLAS SGEMM (TF32 off)" if d.get("bound") == "fp32" else
                            f"{peak_kind} HBM copy"),
            "peaks": pk, "classes": classes,
            "note": "achieved = algorithmic work of the class per step / its event-timed device time per step "
                    "(eager pass over one preconditioner period, graphs off); the gated extra corrections, the "
                    "repeated a' transform and the starting product a0 = X phi' (returning at once on warm starts) "
                    "are the classes extra_corrections, ap_redo and start_product, timed but counted as no work; "
                    "ap_transform is the a' transform, which the graphs run beside the last boundary-sum pass; "
                    "the step is neither HBM- nor tensor-bound: the boundary sums run on the FP32 pipes, "
                    "the transforms on the FP64 pipe"}

    if not args.no_adjoint:
        line["adjoint"] = adjoint_ratio(local_rank)
    if not args.no_batch:
        line["helium_batch"] = helium_batch_summary(args, local_rank, stream)
    if not args.no_cpu:
        rate, cores, times = cpu_sample(3, n)
        line["cpu_baseline"] = {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port",
                                "sample": f"median of 3 RK4 steps at N={n} (FP64 oracle, OpenMP)",
                                "step_s": times}
    print(json.dumps(line), flush=True)


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _state_err(sa, sb, n):
    """max |z_a - z_b| / max |z_b| and the same for phi, from [x|y|phi] arrays."""
    za, zb = sa[:n] + 1j * sa[n:2 * n], sb[:n] + 1j * sb[n:2 * n]
    return [_rel(za, zb), _rel(sa[2 * n:], sb[2 * n:])]


def _empty_graph_ms(kernels: int, replays: int = 50) -> float:
    """Replay time of a CUDA graph of `kernels` dependent one-element kernels:
    the launch-latency floor of a step graph with that many nodes."""
    import torch
    t = torch.zeros(1, device="cuda")
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        t.add_(1.0)  # warm the kernel before capture
    torch.cuda.current_stream().wait_stream(side)
    with torch.cuda.graph(g):
        for _ in range(kernels):
            t.add_(1.0)
    for _ in range(3):
        g.replay()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(replays):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / replays


def run_workload(args, rank, world, local_rank):
    """Secondary workloads (parity and scale cases, one JSON line each):
      modes1024   : gravity wave N=1024, 8 seeded modes (seed 2), dt=0.005,
                    1000 steps mixed; state error vs the FP64 engine every 100
                    steps beside the FP64-vs-perturbed-FP64 envelope (1e-15
                    relative perturbation of x)
      helium-batch: 512 helium films of uneven N (32 * U{4..64}, seed 3),
                    dt=1e-3, 200 steps mixed in one engine per rank (every
                    kernel spans the rank's surfaces, one CUDA graph per step);
                    under torchrun the surfaces are split by LPT on their cost
                    with no collective until the final gather; error vs the
                    FP64 engine after 5 steps; per-surface status
      steep8192   : gravity wave y = 0.3 cos xi, phi = 0.3 sin xi, N=8192,
                    dt=5e-4, 2000 steps mixed; error vs the FP64 engine after
                    10 steps"""
    import torch
    import superfluid_dynamics_gb300 as sfd
    from superfluid_dynamics_gb300 import workloads
    torch.cuda.set_device(local_rank)
    stream = torch.cuda.Stream()
    mixed = sfd.Options(precision=sfd.PRECISION_MIXED, refine_iters=args.refine_iters, pre_iters=args.pre_iters,
                        refactor_every=args.refactor_every, refactor_lag=args.refactor_lag, device=local_rank)
    fp64 = sfd.Options(precision=sfd.PRECISION_FP64, device=local_rank)
    line = {"workload": args.workload, "unit": "steps/s", "higher_is_better": True,
            "config": {"precision": "mixed", "pre_iters": args.pre_iters, "refine_iters": args.refine_iters,
                       "refactor_every": args.refactor_every}}
    if args.workload == "modes1024":
        n, dt, steps = 1024, 0.005, 1000
        s = workloads.random_modes(n, seed=2)
        s0 = np.concatenate([s.x, s.y, s.phi])
        chk = list(range(100, steps + 1, 100))
        res = {}
        for name, opt, eps in (("mixed", mixed, 0.0), ("fp64", fp64, 0.0), ("fp64_perturbed", fp64, 1e-15)):
            eng = sfd.Engine(n, sfd.WaterBoundaryProblem(), opt)
            eng.set_stream(stream.cuda_stream)
            x = s.x * (1 + eps * np.random.default_rng(7).standard_normal(n))
            eng.set_state(x, s.y, s.phi)
            traj, t = [], 0.0
            done = 0
            l0 = eng.kernel_launches
            for c in chk:
                t += _timed_steps(eng, dt, c - done, stream)
                done = c
                traj.append(np.concatenate(eng.get_state()))
            res[name] = (traj, steps / t, eng.status(), (eng.kernel_launches - l0) / steps)
            eng.close()
        line["value"] = res["mixed"][1]
        # latency view: a step against a graph of as many empty dependent kernels
        k = int(round(res["mixed"][3]))
        step_ms = 1e3 / res["mixed"][1]
        line["latency"] = {"step_ms": step_ms, "stage_ms": step_ms / 4, "kernels_per_step": k,
                           "empty_graph_ms": _empty_graph_ms(k)}
        line["fp64_steps_per_s"] = res["fp64"][1]
        line["accuracy"] = {"steps": chk,
                            "mixed_vs_fp64": [_state_err(a, b, n) for a, b in zip(res["mixed"][0], res["fp64"][0])],
                            "fp64_perturbed_vs_fp64": [_state_err(a, b, n) for a, b in
                                                       zip(res["fp64_perturbed"][0], res["fp64"][0])]}
        line["status_or"] = int(np.bitwise_or.reduce(res["mixed"][2][0]))
    elif args.workload == "helium-batch":
        from superfluid_dynamics_gb300 import shard
        allsurfs = workloads.helium_batch(512, seed=3)
        mine = shard.lpt_partition([sf.n for sf in allsurfs], world)[rank]
        surfs = [allsurfs[i] for i in mine]
        ns = [sf.n for sf in surfs]
        phys = [sfd.HeliumBoundaryProblem(depth=sf.depth, A3=sf.A3) for sf in surfs]
        dt, steps = 1e-3, 200
        x = np.concatenate([sf.x for sf in surfs])
        y = np.concatenate([sf.y for sf in surfs])
        ph = np.concatenate([sf.phi for sf in surfs])
        eng = sfd.Engine(ns, phys, mixed)
        eng.set_stream(stream.cuda_stream)
        eng.set_state(x, y, ph)
        _timed_steps(eng, dt, 5, stream)
        m5 = np.concatenate(eng.get_state())
        if world > 1:
            torch.distributed.barrier()
        t = _timed_steps(eng, dt, steps - 5, stream)
        if world > 1:
            tt = torch.tensor([t], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t = float(tt.item())
        st = eng.status()
        line["config"]["sum_groups_per_cta"] = eng.tuning()
        eng.close()
        ref = sfd.Engine(ns, phys, fp64)
        ref.set_state(x, y, ph)
        ref.step(dt, 5)
        f5 = np.concatenate(ref.get_state())
        ref.close()
        nt = sum(ns)
        off = np.concatenate([[0], np.cumsum(ns)])
        errs = [_state_err(np.concatenate([m5[off[i]:off[i + 1]], m5[nt + off[i]:nt + off[i + 1]],
                                           m5[2 * nt + off[i]:2 * nt + off[i + 1]]]),
                           np.concatenate([f5[off[i]:off[i + 1]], f5[nt + off[i]:nt + off[i + 1]],
                                           f5[2 * nt + off[i]:2 * nt + off[i + 1]]]), ns[i]) for i in range(len(ns))]
        local = {g: (int(st[0][k]), errs[k]) for k, g in enumerate(mine)}
        if world > 1:
            allres = shard.gather_states(local, len(allsurfs))
        else:
            allres = [local[i] for i in range(len(allsurfs))]
        if rank != 0:
            return
        flags = np.array([r[0] for r in allres])
        line["value"] = (steps - 5) / t
        line["scaling"] = "strong"
        line["n_gpus"] = world
        line["config"].update({"surfaces": len(allsurfs), "total_nodes": int(sum(sf.n for sf in allsurfs)),
                               "sum_n2": int(sum(sf.n * sf.n for sf in allsurfs)), "dt": dt,
                               "timed_steps": steps - 5,
                               "sharding": f"LPT by N^3 + 2048 N^2 over {world} rank(s), no collective on the data path"})
        line["accuracy"] = {"after_steps": 5, "max_surface_err_z": max(r[1][0] for r in allres),
                            "max_surface_err_phi": max(r[1][1] for r in allres)}
        line["status"] = {"surfaces_nonfinite": int(((flags & sfd._lib.STATUS_NONFINITE) != 0).sum()),
                          "surfaces_pivot_swap": int(((flags & 2) != 0).sum()),
                          "surfaces_refine_stall": int(((flags & 8) != 0).sum())}
    elif args.workload == "steep8192":
        n, dt, steps = 8192, 5e-4, 2000
        s = workloads.linear_wave(n, 0.3)
        eng = sfd.Engine(n, sfd.WaterBoundaryProblem(), mixed)
        eng.set_stream(stream.cuda_stream)
        eng.set_state(s.x, s.y, s.phi)
        _timed_steps(eng, dt, 10, stream)
        m10 = np.concatenate(eng.get_state())
        t = _timed_steps(eng, dt, steps - 10, stream)
        st = eng.status()
        eng.close()
        ref = sfd.Engine(n, sfd.WaterBoundaryProblem(), fp64)
        ref.set_state(s.x, s.y, s.phi)
        t0 = time.perf_counter()
        ref.step(dt, 10)
        t64 = time.perf_counter() - t0
        f10 = np.concatenate(ref.get_state())
        ref.close()
        line["value"] = (steps - 10) / t
        line["fp64_steps_per_s"] = 10 / t64
        line["config"].update({"N": n, "dt": dt, "timed_steps": steps - 10})
        line["accuracy"] = {"after_steps": 10, "mixed_vs_fp64": _state_err(m10, f10, n)}
        line["status_or"] = int(np.bitwise_or.reduce(st[0]))
    else:
        raise SystemExit(f"unknown workload {args.workload}")
    line["metric"] = "RK4 steps/s"
    print(json.dumps(line), flush=True)


def run_profile_window(args, local_rank):
    """The headline engine stepped past its first preconditioner rebuild and
    background switch (60 steps), then --steps steady-state steps between
    cudaProfilerStart and cudaProfilerStop, for captures with
    `ncu --profile-from-start off`.  Prints one informational JSON line."""
    import torch
    import superfluid_dynamics_gb300 as sfd
    from superfluid_dynamics_gb300 import workloads
    torch.cuda.set_device(local_rank)
    s = workloads.random_modes(args.n, seed=2)
    opts = sfd.Options(precision=sfd.PRECISION_MIXED, refine_iters=args.refine_iters,
                       refactor_every=args.refactor_every, pre_iters=args.pre_iters, device=local_rank,
                       refactor_lag=args.refactor_lag, extra_iters=args.extra_iters)
    with sfd.Engine(args.n, sfd.WaterBoundaryProblem(), opts) as eng:
        eng.set_state(s.x, s.y, s.phi)
        eng.step(DT, 60)
        torch.cuda.synchronize()
        l0 = eng.kernel_launches
        torch.cuda.cudart().cudaProfilerStart()
        eng.step(DT, args.steps)
        torch.cuda.synchronize()
        torch.cuda.cudart().cudaProfilerStop()
        print(json.dumps({"workload": "profile window", "N": args.n, "steps": args.steps,
                          "kernel_launches": eng.kernel_launches - l0}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_NODES)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--refine-iters", type=int, default=2)
    ap.add_argument("--pre-iters", type=int, default=2)
    ap.add_argument("--refactor-every", type=int, default=50)
    ap.add_argument("--extra-iters", type=int, default=2,
                    help="gated extra corrections of each solve (run only above the residual tolerance)")
    ap.add_argument("--refactor-lag", type=int, default=8,
                    help="rebuild the preconditioner on a side stream and switch to it this many steps later")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 step and the accuracy study")
    ap.add_argument("--no-batch", action="store_true", help="skip the 512-film helium batch summary")
    ap.add_argument("--no-roofline", action="store_true", help="skip the peak probes and the class roofline")
    ap.add_argument("--precond-fp32", action="store_true", help="apply the preconditioner from FP32 (default FP16 copy)")
    ap.add_argument("--checkpoint-every", type=int, default=50, help="--workload adjoint: checkpoint spacing")
    ap.add_argument("--workload", default="headline",
                    choices=["headline", "modes1024", "helium-batch", "steep8192", "profile", "adjoint"],
                    help="headline = the metric's configuration; the others print their own line")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "profile":
        if rank == 0:
            run_profile_window(args, local_rank)
        return
    if args.workload == "adjoint":  # the fit workload's adjoint alone, --steps RK4 steps
        if rank == 0:
            print(json.dumps(adjoint_ratio(local_rank, args.steps, args.checkpoint_every)), flush=True)
        return
    if args.workload != "headline":
        if world > 1 and args.workload == "helium-batch":
            import torch
            torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
            try:
                run_workload(args, rank, world, local_rank)
            finally:
                torch.distributed.destroy_process_group()
        elif rank == 0:
            run_workload(args, rank, 1, local_rank)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
