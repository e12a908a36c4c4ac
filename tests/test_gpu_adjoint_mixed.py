"""GPU tests of the reverse mode on mixed-precision engines.

A mixed engine records O(n) data per RK4 stage (no LU factors) and solves the
transposed system M^T lambda = ga by FP64 refinement preconditioned with the
transpose of its FP16 approximate inverse.  Its gradients are checked against
the FP64 engine's reverse mode (LU records), which test_gpu_adjoint.py checks
against central finite differences of the CUDA path and of the CPU oracle:
  - one RHS VJP on water, helium (h = 10) and a thin helium film (h = 2) at
    n = 64, 256, 512: gradient within 1e-10 of the FP64 one (relative to its
    largest entry), parameter derivative within 1e-9, no refinement stall;
  - RK4 trajectory VJPs with uneven checkpoint segments: within 1e-8;
  - the fit workload at full size (N=512, 500 steps at dt=1e-3, checkpoints
    every 50): coefficient and A3 gradients within 1e-7;
  - the torch.autograd.Function with precision=PRECISION_MIXED;
  - the captured reverse steps after a parameter change (set_problem) against
    a fresh engine created with the new parameter.
"""
import numpy as np
import pytest

import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import workloads as W
from superfluid_dynamics_gb300._lib import STATUS_REFINE_STALL
from test_gpu_adjoint import CASES, fp64_engine, with_param

pytestmark = pytest.mark.gpu


def mixed_engine(n, phys, every=50):
    return sfd.Engine(n, phys, sfd.Options(precision=sfd.PRECISION_MIXED, pre_iters=2, refactor_every=every,
                                           autotune=False))


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("n", [64, 256, 512])
def test_rhs_vjp_matches_fp64(case, n):
    mk, st = CASES[case]
    phys = mk()
    s = st(n)
    c = np.random.default_rng(31).standard_normal(3 * n)
    with fp64_engine(n, phys) as e:
        g64, gp64 = e.rhs_vjp(s, c)
    with mixed_engine(n, phys) as e:
        e.clear_status()
        g, gp = e.rhs_vjp(s, c)
        status = e.status()[0]
        res, corr = e.adjoint_residual()
    assert res <= 1e-11 and 1 <= corr <= 5, (res, corr)
    assert rel(g, g64) <= 1e-10, rel(g, g64)
    assert abs(gp - gp64) <= 1e-9 * max(abs(gp64), 1e-12), (gp, gp64)
    assert not (status[0] & STATUS_REFINE_STALL), status


@pytest.mark.parametrize("case,dt,steps,every", [("water", 5e-3, 12, 5), ("helium", 1e-3, 30, 7),
                                                 ("helium_h2", 1e-3, 20, 6)])
def test_rk4_vjp_matches_fp64(case, dt, steps, every):
    n = 128
    mk, st = CASES[case]
    phys = mk()
    s = st(n)
    c = np.random.default_rng(41).standard_normal(3 * n)
    with fp64_engine(n, phys) as e:
        f64 = e.rk4_record(dt, steps, every, s)
        g64, gp64 = e.rk4_vjp(c)
    with mixed_engine(n, phys, every=10) as e:
        e.set_state(s[:n], s[n:2 * n] + 1e-3, s[2 * n:])
        x0, y0, p0 = e.get_state()
        e.clear_status()
        f = e.rk4_record(dt, steps, every, s)
        g, gp = e.rk4_vjp(c)
        status = e.status()[0]
        res, corr = e.adjoint_residual()
        assert res <= 1e-11 and 1 <= corr <= 5, (res, corr)
        # the recording leaves the engine's resident state as it was
        x1, y1, p1 = e.get_state()
        assert np.array_equal(x0, x1) and np.array_equal(y0, y1) and np.array_equal(p0, p1)
    assert rel(f, f64) <= 1e-12, rel(f, f64)
    assert rel(g, g64) <= 1e-8, rel(g, g64)
    assert abs(gp - gp64) <= 1e-8 * max(abs(gp64), 1e-12), (gp, gp64)
    assert not (status[0] & STATUS_REFINE_STALL), status


def test_fit_workload_full_size_matches_fp64():
    """The fit workload (N=512, h0=10, A3=1e3, 500 RK4 steps at dt=1e-3,
    checkpoints every 50): the mixed engine's gradient of
    0.5 |y_final - y_target|^2 with respect to the 64 Fourier coefficients and
    A3 against the FP64 engine's."""
    n, steps, dt, every = 512, 500, 1e-3, 50
    s, c0, target = W.helium_fit(n)
    phys = sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3)
    M = c0.size // 2
    m = np.arange(1, M + 1)
    xi = W.nodes(n)
    basis = np.concatenate([np.cos(m[:, None] * xi), np.sin(m[:, None] * xi)])
    state0 = np.concatenate([xi, c0 @ basis, np.zeros(n)])
    out = {}
    for name, mk in (("fp64", lambda: fp64_engine(n, phys)), ("mixed", lambda: mixed_engine(n, phys))):
        with mk() as e:
            f = e.rk4_record(dt, steps, every, state0)
            cot = np.zeros(3 * n)
            cot[n:2 * n] = f[n:2 * n] - target
            g, ga = e.rk4_vjp(cot)
            out[name] = (f, basis @ g[n:2 * n], ga)
    f64, gc64, ga64 = out["fp64"]
    f, gc, ga = out["mixed"]
    assert rel(f, f64) <= 1e-11, rel(f, f64)
    assert rel(gc, gc64) <= 1e-7, rel(gc, gc64)
    assert abs(ga - ga64) <= 1e-7 * abs(ga64), (ga, ga64)


def test_autograd_mixed_matches_fp64():
    torch = pytest.importorskip("torch")
    from superfluid_dynamics_gb300.adjoint import Trajectory, film_state, fourier_basis
    n, steps, dt = 128, 40, 1e-3
    target = torch.from_numpy(W.fourier_surface(n, W.fit_coefficients(40)))
    basis = fourier_basis(n)
    grads = {}
    for prec in (sfd.PRECISION_FP64, sfd.PRECISION_MIXED):
        c0 = torch.from_numpy(W.fit_coefficients(4)).requires_grad_(True)
        a3 = torch.tensor(1e3, dtype=torch.float64, requires_grad=True)
        traj = Trajectory(n, sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3), dt, steps, checkpoint_every=10,
                          precision=prec)
        final = traj(film_state(c0, basis), a3)
        loss = 0.5 * ((final[n:2 * n] - target) ** 2).sum()
        loss.backward()
        grads[prec] = (c0.grad.numpy().copy(), float(a3.grad))
        traj.close()
    gc64, ga64 = grads[sfd.PRECISION_FP64]
    gc, ga = grads[sfd.PRECISION_MIXED]
    assert rel(gc, gc64) <= 1e-8, rel(gc, gc64)
    assert abs(ga - ga64) <= 1e-8 * abs(ga64), (ga, ga64)


def test_captured_steps_follow_set_problem():
    n, dt, steps, every = 128, 1e-3, 12, 5
    mk, st = CASES["helium"]
    phys = mk()
    s = st(n)
    c = np.random.default_rng(51).standard_normal(3 * n)
    phys2 = with_param(phys, 1.5e3)
    with mixed_engine(n, phys) as e:
        e.rk4_record(dt, steps, every, s)
        e.rk4_vjp(c)
        e.set_problem(phys2)
        f = e.rk4_record(dt, steps, every, s)
        g, gp = e.rk4_vjp(c)
    with mixed_engine(n, phys2) as e:
        f2 = e.rk4_record(dt, steps, every, s)
        g2, gp2 = e.rk4_vjp(c)
    assert rel(f, f2) <= 1e-13, rel(f, f2)
    assert rel(g, g2) <= 1e-11, rel(g, g2)
    assert abs(gp - gp2) <= 1e-10 * abs(gp2), (gp, gp2)
