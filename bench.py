"""Benchmark: RK4 steps/s of the Roberts-1983 boundary-integral step on GB300.

Workload (the headline configuration): gravity wave, N = 4096 nodes, 8 seeded
modes (a_m ~ U(0,0.02)/m, theta_m ~ U(0,2 pi), seed 2), phi from the linear
dispersion relation, g = 1, RK4 dt = 0.005, mixed precision (FP32
preconditioner + double-float / FP64 refinement).  Synthetic data: the
reference measures on no dataset.

  value  : steps/s with the state resident in HBM (CUDA events on the engine
           stream around each step; L2 flushed between steps, outside timing)
  e2e    : steps/s through the C ABI with host buffers (pinned host -> device
           copy of the state, one step, device -> host copy, every step)
  roofline: the RK4 step against the tensor roofline of its algorithmic FLOP
           (dense LU + matvecs, bf16 peak / 3); per-kernel-class times from a
           CUDA-event pass over the same workload (graphs off in that pass);
           traffic = DRAM bytes per step from the committed ncu summary
  cpu_baseline: the FP64 CPU oracle (a port of the reference path) on a bounded
           sample (one RK4 step at N = 4096) on this host's cores

--impl reference runs the reference-side CPU path (the oracle port: the
reference's CUDA build needs Windows/MSVC-only pieces and its NumPy calculator
cannot be shipped) on the same workload and prints the same line with
"impl": "reference".  Under torchrun (N > 1) every rank runs an independent
replica (a single surface does not shard); value = all ranks' steps / max time.
"""
from __future__ import annotations

import argparse
import json
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


def step_traffic(n, args):
    """DRAM bytes per RK4 step (read + write, all kernels of one step) from the
    committed ncu summary of this configuration, or None when there is none."""
    key = (f"traffic_bytes_per_step n={n} precision={args.precision} pre_iters={args.pre_iters} "
           f"refine_iters={args.refine_iters} refactor_every={args.refactor_every}:")
    try:
        with open(os.path.join(ROOT, "profiles", "rk4_step_n4096_launches.md")) as f:
            for line in f:
                line = line.strip().strip("`")
                if line.startswith(key):
                    return float(line[len(key):].split()[0])
    except OSError:
        pass
    return None


def adjoint_ratio(device: int):
    """Cost of the hand-written adjoint against the forward pass on the fit
    workload: helium film N=512, h0=10, A3=1e3, 500 RK4 steps at dt=1e-3,
    initial y from 64 seeded Fourier coefficients, checkpoints every 50 steps,
    loss = 0.5 |y_final - y_target|^2.  Forward = the recorded FP64 trajectory
    (sfd_rk4_record); adjoint = sfd_rk4_vjp (segment recomputation with every
    stage recorded, then the reverse sweep).  Wall-clock, synchronous."""
    import superfluid_dynamics_gb300 as sfd
    from superfluid_dynamics_gb300 import workloads
    n, steps, dt, every = 512, 500, 1e-3, 50
    s, c0, target = workloads.helium_fit(n)
    state0 = np.concatenate([s.x, s.y, s.phi])
    eng = sfd.Engine(n, sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3),
                     sfd.Options(precision=sfd.PRECISION_FP64, use_graphs=False, device=device))
    eng.rk4_record(dt, 5, every, state0)          # warm-up (workspace, first launches)
    eng.rk4_vjp(np.zeros(3 * n))
    t0 = time.perf_counter()
    final = eng.rk4_record(dt, steps, every, state0)
    t_fwd = time.perf_counter() - t0
    cot = np.zeros(3 * n)
    cot[n:2 * n] = final[n:2 * n] - target
    t0 = time.perf_counter()
    g, gp = eng.rk4_vjp(cot)
    t_adj = time.perf_counter() - t0
    eng.close()
    return {"workload": "helium film N=512, h0=10, A3=1e3, 500 RK4 steps dt=1e-3, 64 Fourier coefficients, "
                        "checkpoints every 50", "forward_s": t_fwd, "adjoint_s": t_adj, "ratio": t_adj / t_fwd,
            "loss": 0.5 * float(cot[n:2 * n] @ cot[n:2 * n]), "grad_A3": gp}


def cpu_sample(steps: int = 1, n: int = N_NODES):
    """Oracle port (FP64, OpenMP over all host cores): time `steps` RK4 steps."""
    from oracle import oracle
    from superfluid_dynamics_gb300 import workloads
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    s = workloads.random_modes(n, seed=2)
    t0 = time.perf_counter()
    oracle.rk4_steps(oracle.Problem(), s.x, s.y, s.phi, DT, steps)
    dt = time.perf_counter() - t0
    return steps / dt, cores


def run_reference(args, rank, world):
    if rank != 0:
        return
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 2))
    if warm:
        cpu_sample(warm)
    rate, cores = cpu_sample(steps)
    line = {"metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": world, "steps": steps, "warmup": warm,
            "ms_per_step": 1e3 / rate, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded 8-mode gravity wave)", "impl": "reference",
            "config": {"workload": f"gravity wave N={N_NODES}, 8 modes seed 2, RK4 dt={DT}", "N": N_NODES,
                       "precision": "fp64", "path": "CPU FP64 oracle port of the reference RHS + RK4"},
            "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": f"{steps} RK4 step(s) at N={N_NODES} (of the requested {args.steps})"},
            "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch
    import superfluid_dynamics_gb300 as sfd
    from superfluid_dynamics_gb300 import workloads

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    s = workloads.random_modes(args.n, seed=2)
    prec = sfd.PRECISION_MIXED if args.precision == "mixed" else sfd.PRECISION_FP64
    opts = sfd.Options(precision=prec, refine_iters=args.refine_iters, refactor_every=args.refactor_every,
                       pre_iters=args.pre_iters, device=local_rank)
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

    # ---- device-resident timed region
    launches0 = eng.kernel_launches
    times = []
    with ClockSampler(local_rank) as clk:
        with torch.cuda.stream(stream):
            for _ in range(args.steps):
                flush.fill_(1.0)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                eng.step(DT, 1, sync=False)
                e1.record(stream)
                times.append((e0, e1))
            torch.cuda.synchronize()
    gpu_launches = eng.kernel_launches - launches0
    ms = sum(a.elapsed_time(b) for a, b in times)
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

    # ---- end to end through the C ABI with host buffers: every step copies the
    # state in from pinned host memory and the result back out
    x = torch.from_numpy(s.x).pin_memory().numpy()
    y = torch.from_numpy(s.y).pin_memory().numpy()
    p = torch.from_numpy(s.phi).pin_memory().numpy()
    align()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.set_state(x, y, p)
        eng.step(DT, 1)
        x2, y2, p2 = eng.get_state()
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
    per_launch = {name: (tms / cnt, cnt) for name, (tms, cnt) in prof.items() if cnt}
    # Roofline of the step: the dense second-kind solve is a contraction, so the
    # tensor pipe bounds it.  Algorithmic FLOP per RK4 step (one surface):
    #   F(N) = 4 [ (2/3) N^3 (LU) + 2 N^2 (triangular solves) + 2 N^2 (FP64
    #          residual matvec) + 8 N^2 (complex velocity matvec) ]
    # against the bf16 dense peak / 3 (the FP32-equivalent rate of a 3-product
    # bf16 split).  The mixed path replaces most of the LU by a reused FP32
    # preconditioner plus refinement, so this is an equivalent rate.
    flop_step = 4.0 * (2.0 / 3.0 * n ** 3 + 2.0 * n * n + 2.0 * n * n + 8.0 * n * n)
    step_ms = ms / args.steps
    roof = {"bound": "tensor", "kernel": "rk4_step (one CUDA graph launch per step)",
            "achieved": flop_step / (step_ms * 1e-3) / 1e12, "peak": bf16 / 3.0, "unit": "TFLOP/s",
            "algorithmic_flop_per_step": flop_step, "peak_source": f"{peak_kind} bf16 burst / 3"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["traffic"] = step_traffic(n, args)
    roof["classes_ms_per_step"] = {k: round(v[0] * v[1] / prof_steps, 4) for k, v in per_launch.items()}
    dom = max(per_launch, key=lambda k: per_launch[k][0] * per_launch[k][1])
    roof["dominant_class"] = {"name": dom, "avg_launch_ms": round(per_launch[dom][0], 5),
                              "launches_per_step": per_launch[dom][1] / prof_steps}

    adj = None if args.no_adjoint else adjoint_ratio(local_rank)
    cpu = None
    if not args.no_cpu and world >= 1:
        rate, cores = cpu_sample(1, n)
        cpu = {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port",
               "sample": f"1 RK4 step at N={n} (FP64 oracle, OpenMP)"}
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64+df32 (mixed)" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded 8-mode gravity wave)",
            "config": {"workload": f"gravity wave N={n}, 8 modes seed 2, RK4 dt={DT}", "N": n,
                       "precision": args.precision, "refine_iters": args.refine_iters, "pre_iters": args.pre_iters,
                       "refactor_every": args.refactor_every, "l2": "flushed (256 MB write) before every timed step",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": 3 * n * 8,
                    "d2h_bytes_per_step": 3 * n * 8},
            "gpu_launches": gpu_launches, "clocks": clk.summary(), "adjoint": adj}
    print(json.dumps(line), flush=True)


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
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
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
