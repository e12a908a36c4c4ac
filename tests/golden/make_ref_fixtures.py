"""Generate golden fixtures from the reference's own FP64 CUDA path.

Runs the reference harness (oracle/ref_harness.cu, built by oracle/ref_build.sh
from the reference's CuSuperHelium headers) on seeded surfaces and writes one
.npz per case: the inputs x, y, phi, the depth, and the reference's RHS (vx,
vy, dphi) and vortex strength a.  The helium cases pin the oracle's restatement
of createFiniteDepthMKernel (createM.cuh:65-92), createHeliumVelocityMatrices
(WaterVelocities.cuh:72-107) and compute_rhs_helium_phi_expression
(createM.cuh:109-117), with the reference's fixed A3 = h^4 / 3; the water case
cross-checks the fixtures made from the reference's NumPy calculator.  The
harness needs a GPU, so this runs on a GPU machine that holds the reference
sources; the tests only read the .npz outputs.

Usage: python tests/golden/make_ref_fixtures.py --harness oracle/_ref/ref_harness --out tests/golden
       [--time]  also time the reference FP64 RK4 step (water, 8 seeded modes) at N = 1024 and 4096
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from superfluid_dynamics_gb300 import workloads  # noqa: E402


def helium_surface(n, h, seed):
    """A film of depth h with three seeded modes of amplitude up to 0.04 h and
    a small seeded potential."""
    rng = np.random.default_rng(seed)
    xi = workloads.nodes(n)
    y = sum(rng.uniform(0.005, 0.04) * h / m * np.cos(m * xi + rng.uniform(0, 2 * np.pi)) for m in (1, 2, 3))
    phi = sum(rng.uniform(0.0, 0.01) / m * np.sin(m * xi + rng.uniform(0, 2 * np.pi)) for m in (1, 2))
    return xi.copy(), y, phi


CASES = [
    # name, physics, n, depth, surface
    ("ref_helium_n128_h10", "helium", 128, 10.0, lambda: helium_surface(128, 10.0, 101)),
    ("ref_helium_n128_h5", "helium", 128, 5.0, lambda: helium_surface(128, 5.0, 102)),
    ("ref_helium_n256_h8", "helium", 256, 8.0, lambda: helium_surface(256, 8.0, 103)),
    ("ref_water_n128_modes", "water", 128, 1.0,
     lambda: (lambda s: (s.x, s.y, s.phi))(workloads.random_modes(128, seed=2))),
]


def run_rhs(harness, physics, n, depth, x, y, phi, tmp):
    src, dst = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    np.concatenate([x, y, phi]).astype(np.float64).tofile(src)
    subprocess.check_call([harness, "rhs", physics, str(n), repr(depth), src, dst])
    out = np.fromfile(dst, dtype=np.float64)
    return out[:n], out[n:2 * n], out[2 * n:3 * n], out[3 * n:]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--harness", required=True)
    ap.add_argument("--out", required=True)
    ap.add_argument("--time", action="store_true")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        for name, physics, n, depth, make in CASES:
            x, y, phi = make()
            vx, vy, dphi, a = run_rhs(args.harness, physics, n, depth, x, y, phi, tmp)
            np.savez(os.path.join(args.out, name + ".npz"), x=x, y=y, phi=phi, depth=depth, vx=vx, vy=vy,
                     dphi=dphi, a=a)
            print(name, "max|v| %.3e max|dphi| %.3e" % (np.abs(vx + 1j * vy).max(), np.abs(dphi).max()))
        if args.time:
            timing = {}
            for n, steps in ((1024, 10), (4096, 3)):
                s = workloads.random_modes(n, seed=2)
                src = os.path.join(tmp, "in.bin")
                np.concatenate([s.x, s.y, s.phi]).tofile(src)
                out = subprocess.check_output([args.harness, "time", "water", str(n), "1.0", src, str(steps),
                                               "0.005"], text=True)
                f = out.split()
                timing[f"water_modes_n{n}"] = {"steps_per_s": float(f[1]), "ms_per_step": float(f[3]),
                                               "timed_steps": steps}
                print(n, out.strip())
            with open(os.path.join(args.out, "ref_fp64_gpu_step_timing.json"), "w") as fh:
                json.dump(timing, fh, indent=1)


if __name__ == "__main__":
    main()
