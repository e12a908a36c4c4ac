"""The benchmarked solver settings against the oracle.

bench.py times the mixed engine with 2 FP32 pre-iterations, 2 corrections, a
preconditioner rebuilt every 50 steps on a side stream and switched in 8
steps later, CUDA graphs and the autotuned sum shape.  These tests run exactly
those settings and compare with the FP64 oracle (the restatement of the
reference's FP64 step, AutonomousRungeKuttaStepper.cuh:123-307 with
MatrixSolver.cuh:113-172):
  * one RHS of the headline surface (water, N=4096, 8 seeded modes): 1e-10
    of the largest entry;
  * the N=1024 mixed-precision workload over 100 RK4 steps at dt=0.005, which
    crosses two preconditioner rebuilds and one background switch: 1e-10
    relative in z and phi (the FP64 round-off envelope at step 100 is ~3e-15);
  * the uneven helium batch (films of the 512-film workload's generator, seed
    3) over 5 RK4 steps at dt=1e-3 with the batch bench's settings: 1e-10 of
    each surface's largest entry.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

BENCH = dict(precision=sfd.PRECISION_MIXED, pre_iters=2, refine_iters=2, refactor_every=50, refactor_lag=8)


def _threads():
    O.set_threads(os.cpu_count() or 1)


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_headline_rhs_with_bench_settings_matches_oracle():
    _threads()
    n = 4096
    s = W.random_modes(n, seed=2)
    with sfd.Engine(n, sfd.WaterBoundaryProblem(), sfd.Options(**BENCH)) as e:
        e.set_state(s.x, s.y, s.phi)
        dx, dy, dphi = e.rhs()
        st, _, _ = e.status()
        ref = e.refinement()
    (ox, oy, op), _ = O.rhs(O.Problem(), s.x, s.y, s.phi)
    scale = max(np.abs(ox).max(), np.abs(oy).max(), np.abs(op).max())
    err = max(np.abs(dx - ox).max(), np.abs(dy - oy).max(), np.abs(dphi - op).max())
    assert err <= 1e-10 * scale, err / scale
    assert st[0] == 0 and ref["rel_residual"][0] <= 1e-10


def test_modes1024_trajectory_with_bench_settings_matches_oracle():
    _threads()
    n, dt, steps = 1024, 0.005, 100
    s = W.random_modes(n, seed=2)
    with sfd.Engine(n, sfd.WaterBoundaryProblem(), sfd.Options(**BENCH)) as e:
        e.set_state(s.x, s.y, s.phi)
        e.step(dt, steps)
        x, y, phi = e.get_state()
        st, _, _ = e.status()
        ref = e.refinement()
    (rx, ry, rp), _ = O.rk4_steps(O.Problem(), s.x, s.y, s.phi, dt, steps)
    assert _rel(x + 1j * y, rx + 1j * ry) <= 1e-10
    assert _rel(phi, rp) <= 1e-10
    assert st[0] == 0 and ref["stall_rebuilds"] == 0


def test_uneven_helium_batch_with_bench_settings_matches_oracle():
    _threads()
    surfs = W.helium_batch(512, seed=3)[:10]
    dt, steps = 1e-3, 5
    phys = [sfd.HeliumBoundaryProblem(sf.depth, sf.A3) for sf in surfs]
    ns = [sf.n for sf in surfs]
    opt = sfd.Options(precision=sfd.PRECISION_MIXED, pre_iters=2, refine_iters=2, refactor_every=50)
    with sfd.Engine(ns, phys, opt) as e:
        e.set_state(np.concatenate([sf.x for sf in surfs]), np.concatenate([sf.y for sf in surfs]),
                    np.concatenate([sf.phi for sf in surfs]))
        e.step(dt, steps)
        parts = [e.split(v) for v in e.get_state()]
        st, _, _ = e.status()
    for i, sf in enumerate(surfs):
        (rx, ry, rp), _ = O.rk4_steps(O.Problem(physics=O.HELIUM, depth=sf.depth, A3=sf.A3), sf.x, sf.y, sf.phi,
                                      dt, steps)
        scale = max(np.abs(rx).max(), np.abs(ry).max(), np.abs(rp).max())
        err = max(np.abs(parts[0][i] - rx).max(), np.abs(parts[1][i] - ry).max(), np.abs(parts[2][i] - rp).max())
        assert err <= 1e-10 * scale, (i, sf.n, err / scale)
        assert not st[i] & (sfd._lib.STATUS_NONFINITE | sfd._lib.STATUS_ZERO_PIVOT)
