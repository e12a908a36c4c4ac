"""Generate the golden fixtures under tests/golden/ (run in a container that
holds the reference sources; the GPU tests only read the .npz/.json outputs).

Sources of truth:
  * O1 -- the reference's own NumPy calculator, imported unchanged from
    CuSuperHelium/Python/WaterIntegralCalculator.py (+ Derivatives.py):
    water, rho = 0, infinite depth.  Its RHS is evaluated on the seeded
    surfaces below and, for the 128-node linear wave, driven through the
    reference RK4 stage formula (AutonomousRungeKuttaStepper.cuh:123-375).
  * mpmath -- the 50-digit value of cot(0.5 (zk - zj)) at
    zk = pi + i pi, zj = (pi + 0.1) + i (pi + 0.1)
    (the point used by ComplexFunctionsTests.cuh:169-244).

Usage: python tests/golden/make_golden.py [/path/to/reference]
The reference location is the argument, else $SFD_REFERENCE_DIR.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SFD_REFERENCE_DIR", "")
if not REF or not os.path.isdir(REF):
    raise SystemExit("give the reference checkout as the argument or in SFD_REFERENCE_DIR")
sys.path.insert(0, os.path.join(REF, "CuSuperHelium", "Python"))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from WaterIntegralCalculator import WaterIntegralCalculator  # noqa: E402  (reference code)
from superfluid_dynamics_gb300 import workloads  # noqa: E402


def o1_rhs(x, y, phi):
    c = WaterIntegralCalculator()
    c.setInitialState(x, y, phi)
    c.calculateEvolution()
    return dict(vx=np.real(c.vx), vy=np.real(c.vy), dphi=np.real(c.dPhi), a=np.real(c.a),
                xp=np.real(c.Xp), yp=np.real(c.Yp), xpp=np.real(c.Xpp), ypp=np.real(c.Ypp),
                phip=np.real(c.Phip))


def o1_rk4(x, y, phi, dt, steps, keep):
    """RK4 with the reference's stage formula on the state [x, y, phi]."""
    Y0 = np.concatenate([x, y, phi]).astype(np.float64)
    n = x.size
    c = WaterIntegralCalculator()
    f = lambda Y: c.runTimeStep(0.0, Y)  # noqa: E731
    out = {}
    for s in range(1, steps + 1):
        k1 = f(Y0)
        k2 = f(Y0 + dt * 0.5 * k1)
        k3 = f(Y0 + dt * 0.5 * k2)
        k4 = f(Y0 + dt * k3)
        k = k1 + 2.0 * k2 + 2.0 * k3 + k4
        Y0 = Y0 + (dt / 6.0) * k
        if s in keep:
            out[f"x_{s}"], out[f"y_{s}"], out[f"phi_{s}"] = Y0[:n].copy(), Y0[n:2 * n].copy(), Y0[2 * n:].copy()
    return out


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name), **arrays)
    print("wrote", name)


def main():
    # linear wave, 128 nodes (the CPU-runnable configuration)
    s = workloads.linear_wave(128, 0.05)
    save("o1_linear_wave_n128_rhs.npz", x=s.x, y=s.y, phi=s.phi, **o1_rhs(s.x, s.y, s.phi))
    # seeded 8-mode surface at 64 and 256 nodes
    for n in (64, 256):
        s = workloads.random_modes(n, seed=2)
        save(f"o1_modes_seed2_n{n}_rhs.npz", x=s.x, y=s.y, phi=s.phi, **o1_rhs(s.x, s.y, s.phi))
    # steep wave y = 0.3 cos xi at 64 nodes
    s = workloads.linear_wave(64, 0.3)
    save("o1_steep_n64_rhs.npz", x=s.x, y=s.y, phi=s.phi, **o1_rhs(s.x, s.y, s.phi))
    # RK4 trajectory: linear wave, 128 nodes, dt = 0.01, 100 steps
    s = workloads.linear_wave(128, 0.05)
    traj = o1_rk4(s.x, s.y, s.phi, 0.01, 100, keep={1, 10, 100})
    save("o1_linear_wave_n128_rk4.npz", x=s.x, y=s.y, phi=s.phi, dt=np.array(0.01), **traj)
    # 50-digit cotangent
    import mpmath
    mpmath.mp.dps = 50
    zk = mpmath.mpc(mpmath.pi, mpmath.pi)
    zj = mpmath.mpc(mpmath.pi + mpmath.mpf("0.1"), mpmath.pi + mpmath.mpf("0.1"))
    v = mpmath.cot(0.5 * (zk - zj))
    with open(os.path.join(HERE, "cot_50digit.json"), "w") as f:
        json.dump({"zk": [float(zk.real), float(zk.imag)], "zj_offset": 0.1,
                   "cot_re": mpmath.nstr(v.real, 45), "cot_im": mpmath.nstr(v.imag, 45)}, f, indent=1)
    print("wrote cot_50digit.json")


if __name__ == "__main__":
    main()
