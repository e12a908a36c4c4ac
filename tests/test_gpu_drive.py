"""GPU parity of the optomechanically driven helium film (the reference's
HeliumDrivenAutonomousProblem + DelayedIntensityIntegrator, augmented state
[x | y | phi | D]) against the FP64 oracle, and of the SI-unit exports
calculateRhsAugmentedOptomechanical / integrateAugmentedOptomechanicalSimulationRK4.
Tolerances as in test_gpu_parity: FP64 RHS 1e-11, mixed 1e-10 relative to the
largest oracle value; trajectories 1e-9."""
import math

import numpy as np
import pytest

from oracle import oracle as O
import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu
PREC = {"fp64": sfd.PRECISION_FP64, "mixed": sfd.PRECISION_MIXED}
TOL = {"fp64": 1e-11, "mixed": 1e-10}


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def film(n, depth=10.0, seed=8):
    rng = np.random.default_rng(seed)
    xi = W.nodes(n)
    m = np.arange(1, 5)[:, None]
    y = (rng.uniform(0, 0.004 * depth, 4)[:, None] / m * np.cos(m * xi + rng.uniform(0, 6.28, 4)[:, None])).sum(0)
    phi = 0.01 * np.sin(xi)
    D = 0.02 * np.cos(2 * xi)
    return xi, y, phi, D


DRIVE = dict(detuning=0.5, gamma=2.0, G=3.0, tau=5.0, max_intensity=0.4, x0=math.pi, sigma=0.6, beta=0.2,
             damping=0.05, strength=0.3)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("n,augmented", [(64, True), (512, True), (96, False)])
def test_driven_rhs_matches_oracle(prec, n, augmented):
    x, y, phi, D = film(n)
    phys = sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3)
    drv = sfd.Drive(augmented=augmented, **DRIVE)
    with sfd.Engine(n, phys, sfd.Options(precision=PREC[prec]), drive=drv) as e:
        e.set_state(x, y, phi)
        if augmented:
            e.set_aux(D)
        import torch
        st = torch.tensor(np.concatenate([x, y, phi] + ([D] if augmented else [])), device="cuda")
        out = torch.empty_like(st)
        e.rhs_device(st.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        got = out.cpu().numpy()
    ref, _ = O.rhs_driven(O.Problem(physics=sfd.HELIUM, depth=10.0, A3=1e3), O.Drive(augmented=augmented, **DRIVE),
                          x, y, phi, D)
    assert rel(got[:n] + 1j * got[n:2 * n], ref[0] + 1j * ref[1]) < TOL[prec]
    assert rel(got[2 * n:3 * n], ref[2]) < TOL[prec]
    if augmented:
        assert rel(got[3 * n:], ref[3]) < TOL[prec]
    # the drive changes dphi by more than the tolerance
    plain, _ = O.rhs(O.Problem(physics=sfd.HELIUM, depth=10.0, A3=1e3), x, y, phi)
    assert np.abs(ref[2] - plain[2]).max() > 1e-3 * np.abs(ref[2]).max()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_augmented_rk4_matches_oracle(prec):
    n, dt, steps = 128, 2e-3, 25
    x, y, phi, D = film(n, seed=9)
    phys = sfd.HeliumBoundaryProblem(depth=10.0, A3=1e3)
    with sfd.Engine(n, phys, sfd.Options(precision=PREC[prec]), drive=sfd.Drive(**DRIVE)) as e:
        e.set_state(x, y, phi)
        e.set_aux(D)
        e.step(dt, steps)
        gx, gy, gp = e.get_state()
        gD = e.get_aux()
    (ox, oy, op, oD), _ = O.rk4_steps_driven(O.Problem(physics=sfd.HELIUM, depth=10.0, A3=1e3),
                                             O.Drive(**DRIVE), x, y, phi, D, dt, steps)
    assert rel(gx + 1j * gy, ox + 1j * oy) < 1e-9
    assert rel(gp, op) < 1e-9
    assert rel(gD, oD) < 1e-9
    assert rel(oD, D) > 1e-6  # D evolved


def nondim(sp, ov):
    """Restates adimensionalizeProperties / adimensionalizeOptomechanicalVariables
    (Export.cu:1222-1270) and the drive prefactor (LightIntensity.cuh:34-37) for
    the checker."""
    hbar, alpha, rho_he = 1.054571817e-34, 3.5e-24, 150.0
    Lb = sp.L / (2 * math.pi)
    acc = 3 * alpha / sp.depth ** 4
    Tb = math.sqrt(Lb / acc)
    Eb = 3.0 * rho_he * alpha * Lb ** 4 / sp.depth ** 4
    rho = sp.rho / rho_he
    depth = sp.depth / Lb
    G = ov.G * Tb * Lb
    tau = ov.tau / Tb
    sigma = ov.sigma_optical_mode / Lb
    beta = ov.beta * (hbar / Eb / Tb) * G / tau / (sigma ** 2 * rho)
    d = O.Drive(detuning=ov.detuning * Tb, gamma=ov.gamma * Tb, G=G, tau=tau, max_intensity=ov.max_intensity,
                x0=ov.location_x0_mode / Lb, sigma=sigma, beta=beta, damping=ov.damping_strength,
                strength=hbar / (Eb * Tb * rho) * G / sigma ** 2, augmented=True)
    return O.Problem(physics=sfd.HELIUM, depth=depth), d, Tb


def si_case(n):
    # film and cavity of the reference's augmented-RHS study (1 um period, 15 nm film), with the drive
    # strengths raised so that every drive term shows in the result
    sp = _lib.SimProperties(L=1e-6, rho=150.0, kappa=0.0, depth=15e-9, use_expansions=False, expansion_order=1,
                            infinite_depth=False)
    ov = _lib.COptomechanicalVariables(detuning=3e7, gamma=5e7, G=2e14, tau=1e-6, max_intensity=1e9,
                                       initial_time=0.0, location_x0_mode=5e-7, sigma_optical_mode=1e-7,
                                       beta=1e3, damping_strength=0.05)
    prob, drv, Tb = nondim(sp, ov)
    xi = W.nodes(n)
    y = 0.05 * prob.depth * np.cos(2 * xi)
    state = np.concatenate([xi, y, 0.001 * np.sin(xi), 1e-3 * np.cos(xi)])
    return sp, ov, prob, drv, Tb, state


def test_augmented_rhs_export_matches_oracle():
    n = 128
    sp, ov, prob, drv, Tb, state = si_case(n)
    got = sfd.SimulationManager().calculate_augmented_rhs(state, sp, ov)
    ref, _ = O.rhs_driven(prob, drv, state[:n], state[n:2 * n], state[2 * n:3 * n], state[3 * n:])
    assert rel(got[:n] + 1j * got[n:2 * n], ref[0] + 1j * ref[1]) < 1e-11
    assert rel(got[2 * n:3 * n], ref[2]) < 1e-11
    assert rel(got[3 * n:], ref[3]) < 1e-11


def test_augmented_rk4_export_matches_oracle():
    n = 64
    sp, ov, prob, drv, Tb, state = si_case(n)
    dt_nd, steps = 1e-3, 12
    ro = _lib.RK4SolverOptions(timeStep=dt_nd * Tb, t0=0.0, t1=(steps + 0.5) * dt_nd * Tb, returnTrajectory=True)
    rc, T, S = sfd.SimulationManager().integrate_augmented_optomechanical_problem(state, sp, ov, ro)
    assert rc == 0 and S.shape == (steps + 1, 4 * n) and T.size == steps + 1
    assert np.array_equal(S[0], state)
    (ox, oy, op, oD), _ = O.rk4_steps_driven(prob, drv, state[:n], state[n:2 * n], state[2 * n:3 * n],
                                             state[3 * n:], dt_nd, steps)
    f = S[-1]
    assert rel(f[:n] + 1j * f[n:2 * n], ox + 1j * oy) < 1e-9
    assert rel(f[2 * n:3 * n], op) < 1e-9
    assert rel(f[3 * n:], oD) < 1e-9
