"""GPU tests of the hand-written adjoint (reverse mode) of the FP64 RHS and of
RK4 trajectories.

Checks, each on seeded surfaces:
  - dot-product test of the RHS VJP against central finite differences of the
    CUDA forward path (h = 1e-6): |<c, J v>_FD - <J^T c, v>| <= 1e-6 relative,
    for the state and for the parameter (A3 helium, g water);
  - RK4 trajectory VJP (uneven checkpoint segments) against central finite
    differences of the CUDA forward path, and against finite differences of the
    FP64 CPU oracle (the reference gradient) on a small case;
  - the torch.autograd.Function over the fit workload's Fourier coefficients.
"""
import numpy as np
import pytest

from oracle import oracle as O
import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import workloads as W

pytestmark = pytest.mark.gpu
FD_H = 1e-6


def fp64_engine(n, phys):
    # autotune off: the tuner times the sum shapes on the first step() and the
    # shape it keeps sets the summation order, so a trajectory recorded before
    # it ran could differ from the steps in the last bits
    return sfd.Engine(n, phys, sfd.Options(precision=sfd.PRECISION_FP64, use_graphs=False, autotune=False))


def rhs_of(e, state, n):
    e.set_state(state[:n], state[n:2 * n], state[2 * n:])
    dx, dy, dphi = e.rhs()
    return np.concatenate([dx, dy, dphi])


def film(n, seed, depth=10.0):
    """A film with six seeded modes of amplitude up to 0.5 % of the depth and a small potential."""
    rng = np.random.default_rng(seed)
    xi = W.nodes(n)
    m = np.arange(1, 7)[:, None]
    amp = rng.uniform(0.0, 0.005 * depth, 6)[:, None] / m
    th = rng.uniform(0.0, 2 * np.pi, 6)[:, None]
    y = (amp * np.cos(m * xi + th)).sum(0)
    phi = 0.01 * np.sin(2 * xi)
    return np.concatenate([xi, y, phi])


CASES = {
    "water": (lambda: sfd.WaterBoundaryProblem(), lambda n: np.concatenate(
        [W.random_modes(n, seed=2).x, W.random_modes(n, seed=2).y, W.random_modes(n, seed=2).phi])),
    "helium": (lambda: sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3), lambda n: film(n, 5)),
    "helium_h2": (lambda: sfd.HeliumBoundaryProblem(depth=2.0, A3=3.0), lambda n: film(n, 6, depth=2.0)),
}


def with_param(phys, v):
    import dataclasses
    f = {k.name: getattr(phys, k.name) for k in dataclasses.fields(sfd.Physics)}
    f["A3" if phys.physics == sfd.HELIUM else "gravity"] = v
    return sfd.Physics(**f)


def param_of(phys):
    return phys.A3 if phys.physics == sfd.HELIUM else phys.gravity


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("n", [64, 128])
def test_rhs_vjp_dot_product(case, n):
    mk, st = CASES[case]
    phys = mk()
    s = st(n)
    rng = np.random.default_rng(11)
    c = rng.standard_normal(3 * n)
    v = rng.standard_normal(3 * n) * np.concatenate([np.full(n, 1e-2), np.full(n, 1e-2), np.full(n, 1e-2)])
    with fp64_engine(n, phys) as e:
        g, gp = e.rhs_vjp(s, c)
        fp = rhs_of(e, s + FD_H * v, n)
        fm = rhs_of(e, s - FD_H * v, n)
        fd = c @ (fp - fm) / (2 * FD_H)
        ad = g @ v
        assert abs(fd - ad) <= 1e-6 * max(abs(fd), np.abs(c).max() * 1e-3), (fd, ad)
        # parameter
        p0 = param_of(phys)
        hp = 1e-6 * abs(p0)
        e.set_problem(with_param(phys, p0 + hp))
        fp = rhs_of(e, s, n)
        e.set_problem(with_param(phys, p0 - hp))
        fm = rhs_of(e, s, n)
        e.set_problem(phys)
        fdp = c @ (fp - fm) / (2 * hp)
        assert abs(fdp - gp) <= 1e-6 * max(abs(fdp), 1e-12), (fdp, gp)


@pytest.mark.parametrize("case", ["water", "helium"])
def test_rhs_vjp_components(case):
    """Per-component check: unit cotangents on a few outputs, unit directions on
    a few inputs (catches errors that cancel in a random dot product)."""
    n = 64
    mk, st = CASES[case]
    phys = mk()
    s = st(n)
    with fp64_engine(n, phys) as e:
        for out_idx in (3, n + 17, 2 * n + 40):
            c = np.zeros(3 * n)
            c[out_idx] = 1.0
            g, _ = e.rhs_vjp(s, c)
            for in_idx in (5, n + 9, 2 * n + 33, out_idx % n, n + out_idx % n):
                v = np.zeros(3 * n)
                v[in_idx] = 1.0
                fd = (rhs_of(e, s + FD_H * v, n)[out_idx] - rhs_of(e, s - FD_H * v, n)[out_idx]) / (2 * FD_H)
                assert abs(fd - g[in_idx]) <= 2e-6 * max(abs(fd), 1e-3), (out_idx, in_idx, fd, g[in_idx])


def traj_final(e, state0, dt, steps):
    return e.rk4_record(dt, steps, max(1, steps), state0)


@pytest.mark.parametrize("case,dt,steps,every", [("water", 5e-3, 12, 5), ("helium", 1e-3, 10, 3)])
def test_rk4_vjp_vs_fd(case, dt, steps, every):
    n = 64
    mk, st = CASES[case]
    phys = mk()
    s = st(n)
    rng = np.random.default_rng(21)
    c = rng.standard_normal(3 * n)
    v = 1e-2 * rng.standard_normal(3 * n)
    with fp64_engine(n, phys) as e:
        final = e.rk4_record(dt, steps, every, s)
        # the recorded trajectory equals the engine's own RK4 steps
        e.set_state(s[:n], s[n:2 * n], s[2 * n:])
        e.step(dt, steps)
        assert np.array_equal(np.concatenate(e.get_state()), final)
        g, gp = e.rk4_vjp(c)
        fp = traj_final(e, s + FD_H * v, dt, steps)
        fm = traj_final(e, s - FD_H * v, dt, steps)
        fd = c @ (fp - fm) / (2 * FD_H)
        assert abs(fd - g @ v) <= 1e-6 * abs(fd), (fd, g @ v)
        p0 = param_of(phys)
        hp = 1e-6 * abs(p0)
        e.set_problem(with_param(phys, p0 + hp))
        fp = traj_final(e, s, dt, steps)
        e.set_problem(with_param(phys, p0 - hp))
        fm = traj_final(e, s, dt, steps)
        e.set_problem(phys)
        fdp = c @ (fp - fm) / (2 * hp)
        assert abs(fdp - gp) <= 1e-5 * max(abs(fdp), 1e-12), (fdp, gp)


def test_rk4_vjp_vs_oracle_gradient():
    """Reference gradient: central differences of the FP64 CPU oracle."""
    n, dt, steps = 32, 1e-3, 6
    phys = sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3)
    s = film(n, 7)
    op = O.Problem(physics=phys.physics, depth=phys.depth, A3=phys.A3)
    c = np.zeros(3 * n)
    c[n:2 * n] = np.random.default_rng(3).standard_normal(n)     # loss on y only
    with fp64_engine(n, phys) as e:
        e.rk4_record(dt, steps, 4, s)
        g, _ = e.rk4_vjp(c)
    for idx in (2, n + 5, n + 20, 2 * n + 11):
        sp, sm = s.copy(), s.copy()
        sp[idx] += FD_H
        sm[idx] -= FD_H
        fp = np.concatenate(O.rk4_steps(op, sp[:n], sp[n:2 * n], sp[2 * n:], dt, steps)[0])
        fm = np.concatenate(O.rk4_steps(op, sm[:n], sm[n:2 * n], sm[2 * n:], dt, steps)[0])
        fd = c @ (fp - fm) / (2 * FD_H)
        assert abs(fd - g[idx]) <= 1e-6 * max(abs(fd), 1e-4), (idx, fd, g[idx])


def test_autograd_fourier_fit():
    """torch.autograd over the fit workload (64 Fourier coefficients + A3) at a
    reduced size: N = 128, 40 steps, checkpoints every 10."""
    torch = pytest.importorskip("torch")
    from superfluid_dynamics_gb300.adjoint import Trajectory, fourier_basis, film_state
    n, steps, dt = 128, 40, 1e-3
    c0 = torch.from_numpy(W.fit_coefficients(4)).requires_grad_(True)
    a3 = torch.tensor(1e3, dtype=torch.float64, requires_grad=True)
    target = torch.from_numpy(W.fourier_surface(n, W.fit_coefficients(40)))
    basis = fourier_basis(n)
    traj = Trajectory(n, sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3), dt, steps, checkpoint_every=10)

    def loss_of(coeffs, a3v):
        final = traj(film_state(coeffs, basis), a3v)
        return 0.5 * ((final[n:2 * n] - target) ** 2).sum()

    loss = loss_of(c0, a3)
    loss.backward()
    gc, ga = c0.grad.clone(), float(a3.grad)
    with torch.no_grad():
        for i in (0, 7, 33, 63):
            e = torch.zeros_like(c0)
            e[i] = FD_H
            fd = (float(loss_of(c0 + e, a3)) - float(loss_of(c0 - e, a3))) / (2 * FD_H)
            assert abs(fd - float(gc[i])) <= 1e-5 * max(abs(fd), 1e-8), (i, fd, float(gc[i]))
        h = 1e-6 * 1e3
        fd = (float(loss_of(c0, a3 + h)) - float(loss_of(c0, a3 - h))) / (2 * h)
        assert abs(fd - ga) <= 1e-5 * max(abs(fd), 1e-14), (fd, ga)
    traj.close()


def test_fit_workload_full_size_gradient():
    """The fit workload at full size (N=512, h0=10, A3=1e3, 500 steps at
    dt=1e-3, checkpoints every 50): adjoint gradient of the loss
    0.5 |y_final - y_target|^2 against central differences (h = 1e-6) for
    three Fourier coefficients and A3."""
    n, steps, dt, every = 512, 500, 1e-3, 50
    s, c0, target = W.helium_fit(n)
    phys = sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3)
    M = c0.size // 2
    m = np.arange(1, M + 1)
    xi = W.nodes(n)
    basis = np.concatenate([np.cos(m[:, None] * xi), np.sin(m[:, None] * xi)])

    def state_of(c):
        return np.concatenate([xi, c @ basis, np.zeros(n)])

    with fp64_engine(n, phys) as e:
        def loss(c, a3=1e3):
            e.set_problem(with_param(phys, a3))
            f = e.rk4_record(dt, steps, every, state_of(c))
            return 0.5 * float(((f[n:2 * n] - target) ** 2).sum()), f

        L0, f0 = loss(c0)
        cot = np.zeros(3 * n)
        cot[n:2 * n] = f0[n:2 * n] - target
        g, ga = e.rk4_vjp(cot)
        gc = basis @ g[n:2 * n]
        for i in (0, 20, 45):
            d = np.zeros_like(c0)
            d[i] = FD_H
            fd = (loss(c0 + d)[0] - loss(c0 - d)[0]) / (2 * FD_H)
            assert abs(fd - gc[i]) <= 1e-5 * max(abs(fd), 1e-10), (i, fd, gc[i])
        h = 1e-6 * 1e3
        fd = (loss(c0, 1e3 + h)[0] - loss(c0, 1e3 - h)[0]) / (2 * h)
        assert abs(fd - ga) <= 1e-5 * max(abs(fd), 1e-16), (fd, ga)
