"""GPU parity of the adaptive Runge-Kutta-Fehlberg 4(5) integrator (the
reference's RK45Base) against its CPU restatement in the oracle: the same
accepted / rejected step sequence, the final state to 1e-9 relative, and the
step times to 1e-8 (the error estimate is a difference of stage slopes of
size ~tol, so its round-off differs between GPU and oracle by up to ~1e-5
relative at tol = 1e-12, and the step factor goes as err^(-1/5))."""
import numpy as np
import pytest

from oracle import oracle as O
import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.mark.parametrize("prec", [sfd.PRECISION_FP64, sfd.PRECISION_MIXED])
@pytest.mark.parametrize("case", ["water", "helium"])
def test_rkf45_matches_oracle(prec, case):
    n = 64
    if case == "water":
        s = W.linear_wave(n, 0.08)
        phys, op = sfd.WaterBoundaryProblem(), O.Problem()
        t1, tol = 1.5, (1e-9, 1e-7)
    else:
        s = W.random_modes(n, seed=5)
        phys = sfd.HeliumBoundaryProblem(depth=2.0, A3=3.0)
        op = O.Problem(physics=sfd.HELIUM, depth=2.0, A3=3.0)
        t1, tol = 1.0, (1e-12, 1e-10)
    with sfd.Engine(n, phys, sfd.Options(precision=prec, use_graphs=False)) as e:
        e.set_state(s.x, s.y, s.phi)
        res, times = e.evolve_rkf45(0.0, t1, atol=tol[0], rtol=tol[1], h0=0.05)
        gx, gy, gp = e.get_state()
    (ox, oy, ophi), st, t, h, acc, rej, otimes = O.rkf45_evolve(op, s.x, s.y, s.phi, 0.0, t1, atol=tol[0],
                                                                 rtol=tol[1], h0=0.05)
    assert res["status"] == st == 0
    assert res["accepted"] == acc and res["rejected"] == rej and acc > 3
    assert rel(times, otimes) < 1e-8
    assert abs(res["t"] - t) < 1e-12 and abs(res["h"] - h) < 1e-6 * abs(h)
    assert rel(gx + 1j * gy, ox + 1j * oy) < 1e-9
    assert rel(gp, ophi) < 1e-9


def test_rkf45_reports_rejections_and_reaches_t1():
    n = 32
    s = W.linear_wave(n, 0.1)
    with sfd.Engine(n, sfd.WaterBoundaryProblem(), sfd.Options(precision=sfd.PRECISION_FP64)) as e:
        e.set_state(s.x, s.y, s.phi)
        res, times = e.evolve_rkf45(0.0, 0.7, atol=1e-12, rtol=1e-10, h0=1.0)  # far too large a first step
    assert res["status"] == 0 and res["rejected"] >= 1
    assert abs(times[-1] - 0.7) < 1e-14 and abs(res["t"] - 0.7) < 1e-14
