"""Time the reference's own CPU path: its NumPy water calculator
(CuSuperHelium/Python/WaterIntegralCalculator.py:7-84 with Derivatives.py),
imported unchanged, one RHS evaluation per call, on the seeded 8-mode water
surface of the benchmarks.  The reference checkout exists only on the build
machine, so this runs there and commits its numbers (with the host it ran
on) to tests/golden/ref_numpy_rhs_timing.json; nothing reads the reference at
test or bench time.

Usage: python tests/golden/time_reference_numpy.py [/path/to/reference]
The reference location is the argument, else $SFD_REFERENCE_DIR.
"""
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SFD_REFERENCE_DIR", "")
if not REF or not os.path.isdir(REF):
    raise SystemExit("give the reference checkout as the argument or in SFD_REFERENCE_DIR")
sys.path.insert(0, os.path.join(REF, "CuSuperHelium", "Python"))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from WaterIntegralCalculator import WaterIntegralCalculator  # noqa: E402  (reference code)
from superfluid_dynamics_gb300 import workloads  # noqa: E402


def rhs_seconds(n, reps):
    s = workloads.random_modes(n, seed=2)
    out = []
    for _ in range(reps):
        c = WaterIntegralCalculator()
        t0 = time.perf_counter()
        c.setInitialState(s.x, s.y, s.phi)
        c.calculateEvolution()
        out.append(time.perf_counter() - t0)
    return out


def main():
    res = {"host": {"machine": platform.machine(), "processor": platform.processor() or platform.machine(),
                    "cpus": os.cpu_count(), "numpy": np.__version__},
           "workload": "water, 8 seeded modes (seed 2), one RHS evaluation per call; an RK4 step is 4 of them"}
    for n, reps in ((128, 5), (256, 5), (1024, 3)):
        t = rhs_seconds(n, reps)
        med = float(np.median(t))
        res[f"n{n}"] = {"rhs_s_median": med, "rhs_s": t, "rk4_steps_per_s": 1.0 / (4 * med)}
        print(n, "median RHS %.4f s, RK4 %.3f steps/s" % (med, 1.0 / (4 * med)))
    with open(os.path.join(HERE, "ref_numpy_rhs_timing.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
