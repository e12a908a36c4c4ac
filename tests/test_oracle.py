"""CPU tests: pin the FP64 oracle against the reference's own NumPy calculator
(golden fixtures made by tests/golden/make_golden.py) and against the
known-answer tests of the reference's gtest suite, re-derived here:
  MatrixMTests.cuh:69-87,160-223   closed-form 2x2 M
  MatrixMTests.cuh:89-115,225-282  M at N=4 vs a host restatement
  MatrixMTests.cuh:117-151,396-468 V1, V2 at N=8
  MatrixMTests.cuh:51-67,477-607   spectral derivatives of a Lagrangian Stokes wave, N=1024
  MatrixMTests.cuh:735-820         water Bernoulli, N=32
  ComplexFunctionsTests.cuh:169-244 cot Green's function vs a 50-digit value
and against outputs of the reference's own FP64 CUDA path (fixtures made by
tests/golden/make_ref_fixtures.py with oracle/ref_harness.cu): finite-depth
helium films (createFiniteDepthMKernel, createHeliumVelocityMatrices,
compute_rhs_helium_phi_expression with A3 = h^4/3) and a water surface.
"""
import cmath
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


# --- Lagrangian Stokes wave of MatrixMTests.cuh:19-67 (per-index derivatives)
def stokes(N, h, omega, t, rho=0.0):
    j = 2 * np.pi * np.arange(N) / N
    X = j - h * np.sin(j - omega * t)
    Y = h * np.cos(j - omega * t)
    Phi = h * (1 + rho) * omega * np.sin(j - omega * t)
    s1, s2 = 2 * np.pi / N, 4 * np.pi ** 2 / N ** 2
    Zp = s1 * ((1 - h * np.cos(j - omega * t)) + 1j * (-h * np.sin(j - omega * t)))
    Zpp = s2 * ((h * np.sin(j - omega * t)) + 1j * (-h * np.cos(j - omega * t)))
    PhiP = s1 * h * (1 + rho) * omega * np.cos(j - omega * t)
    return X + 1j * Y, Phi, Zp, Zpp, PhiP


@pytest.mark.parametrize("name", ["o1_linear_wave_n128_rhs", "o1_modes_seed2_n64_rhs",
                                  "o1_modes_seed2_n256_rhs", "o1_steep_n64_rhs"])
def test_oracle_rhs_matches_reference_numpy(name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    (dx, dy, dphi, a, zp, zpp), info = O.rhs(O.Problem(), d["x"], d["y"], d["phi"], diagnostics=True)
    assert info == 0
    # the reference NumPy code treats the Nyquist mode differently from the CUDA
    # path (Derivatives.py:13-17 vs utilities.cuh:126-141): agreement ~1e-14
    vel = dx + 1j * dy
    for got, ref in [(vel, d["vx"] + 1j * d["vy"]), (dphi, d["dphi"]), (a, d["a"]),
                     (zp, d["xp"] + 1j * d["yp"]), (zpp, d["xpp"] + 1j * d["ypp"])]:
        assert rel(got, ref) < 1e-11


def test_oracle_rk4_matches_reference_numpy():
    d = np.load(os.path.join(GOLD, "o1_linear_wave_n128_rk4.npz"))
    for steps in (1, 10, 100):
        (x, y, phi), info = O.rk4_steps(O.Problem(), d["x"], d["y"], d["phi"], float(d["dt"]), steps)
        assert info == 0
        assert np.abs(x - d[f"x_{steps}"]).max() < 1e-13
        assert np.abs(y - d[f"y_{steps}"]).max() < 1e-13
        assert np.abs(phi - d[f"phi_{steps}"]).max() < 1e-13


def test_two_by_two_M_closed_form():
    h = 0.5
    Z, _, Zp, Zpp, _ = stokes(2, h, 10.0, 0.0)
    M = O.create_M(O.Problem(), Z, Zp, Zpp)
    expect = np.array([[0.5 - 0.25 * h / (1 - h), (h - 1) / 4 * math.sinh(2 * h) / (math.cosh(2 * h) + 1)],
                       [(h + 1) / 4 * math.sinh(2 * h) / (math.cosh(2 * h) + 1), 0.5 + 0.25 * h / (1 + h)]])
    assert np.abs(M - expect).max() < 1e-14


def test_M_n4_host_restatement():
    N, h, om, t = 4, 0.5, 10.0, 0.1
    Z, _, Zp, Zpp, _ = stokes(N, h, om, t)
    M = O.create_M(O.Problem(), Z, Zp, Zpp)
    for k in range(N):
        for j in range(N):
            if k == j:
                e = 0.5 + 0.25 / math.pi * (Zpp[k] / Zp[k]).imag
            else:
                e = 0.25 / math.pi * (Zp[k] / cmath.tan(0.5 * (Z[k] - Z[j]))).imag
            assert abs(M[k, j] - e) < 1e-14


def test_velocity_n8_host_restatement():
    N, h, om, t = 8, 0.5, 10.0, 0.1
    Z, _, Zp, Zpp, _ = stokes(N, h, om, t)
    rng = np.random.default_rng(8)
    a = rng.standard_normal(N)
    ap = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    V1 = np.empty((N, N), complex)
    V2 = np.empty(N, complex)
    for k in range(N):
        for j in range(N):
            if k == j:
                V1[k, j] = -0.25j / math.pi * Zpp[k] / Zp[k] ** 2 + 0.5 / Zp[k]
                V2[k] = 0.5j / (math.pi * Zp[k])
            else:
                V1[k, j] = -0.25j / math.pi / cmath.tan(0.5 * (Z[k] - Z[j]))
    expect = np.conj(V1 @ a + V2 * ap)
    vel = O.velocities(O.Problem(), Z, Zp, Zpp, a, ap)
    assert rel(vel, expect) < 1e-13


def test_stokes_derivatives_n1024():
    N = 1024
    Z, Phi, Zp, Zpp, PhiP = stokes(N, 0.5, 10.0, 0.0)
    zp, php, zpp = O.zphi_derivative(Z, Phi.astype(complex))
    assert np.abs(zp - Zp).max() < 1e-14
    assert np.abs(zpp - Zpp).max() < 1e-14
    assert np.abs(php.real - PhiP).max() < 1e-14


def test_water_bernoulli_n32():
    N, h, om, t = 32, 0.5, 10.0, 0.1
    rng = np.random.default_rng(32)
    Z = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    v = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    out = O.rhs_phi_water(Z, v, np.zeros(N, complex), 0.0, 1.0)
    assert np.abs(out - (-Z.imag + 0.5 * np.abs(v) ** 2)).max() < 1e-14


def test_cot_green_50_digits():
    d = json.load(open(os.path.join(GOLD, "cot_50digit.json")))
    zk = complex(math.pi, math.pi)
    zj = complex(math.pi + 0.1, math.pi + 0.1)
    v = O.cot_green(zk, zj)
    assert abs(v.real - float(d["cot_re"])) < 1e-13
    assert abs(v.imag - float(d["cot_im"])) < 1e-13


@pytest.mark.parametrize("n", [8, 96, 128, 160, 32 * 61, 1024])
def test_fft_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert rel(O.fft(x), np.fft.fft(x)) < 1e-14
    assert rel(O.fft(x, inverse=True), np.fft.ifft(x) * n) < 1e-14


def test_lu_solve_matches_numpy():
    rng = np.random.default_rng(1)
    A = rng.standard_normal((200, 200)) + 10 * np.eye(200)
    b = rng.standard_normal(200)
    x, info = O.lu_solve(A, b)
    assert info == 0
    assert rel(x, np.linalg.solve(A, b)) < 1e-12


def test_helium_flat_film_is_stationary():
    # flat film, phi = 0: the van der Waals offset makes dphi/dt = 0 and v = 0
    N = 64
    xi = 2 * np.pi * np.arange(N) / N
    for A3 in (None, 1e3):
        (dx, dy, dphi), info = O.rhs(O.Problem(physics=O.HELIUM, depth=10.0, A3=A3), xi, 0 * xi, 0 * xi)
        assert info == 0
        assert np.abs(dphi).max() < 1e-12 and np.abs(dy).max() < 1e-12


def test_oracle_drive_terms_known_answers():
    """Driven film (CSH/createM.cuh:141-178, LightIntensity.cuh:25-37): on a
    flat film at rest the base RHS vanishes, so dphi is exactly
    strength * I + D and dD = beta * I - D / tau; I at the mode centre with
    G y = 0 is gamma^2 I_max / 4 / (detuning^2 + gamma^2 / 4)."""
    n = 32
    xi = 2 * np.pi * np.arange(n) / n
    P = O.Problem(physics=O.HELIUM, depth=3.0)
    d = O.Drive(detuning=0.4, gamma=1.2, G=2.0, tau=3.0, max_intensity=0.5, x0=xi[7], sigma=0.3, beta=0.7,
                damping=0.2, strength=1.5, augmented=True)
    D = 0.1 * np.cos(xi)
    (dx, dy, dphi, dD), info = O.rhs_driven(P, d, xi, np.zeros(n), np.zeros(n), D)
    inten = 0.25 * d.gamma ** 2 * d.max_intensity / (d.detuning ** 2 + (d.gamma / 2) ** 2) * \
        np.exp(-(xi - d.x0) ** 2 / (2 * d.sigma ** 2))
    assert info == 0
    assert np.abs(dx).max() < 1e-14 and np.abs(dy).max() < 1e-14
    assert np.allclose(dphi, d.strength * inten + D, rtol=0, atol=1e-14)
    assert np.allclose(dD, d.beta * inten - D / d.tau, rtol=0, atol=1e-14)
    # without augmentation D is neither read nor produced
    (dx2, dy2, dphi2), _ = O.rhs_driven(P, O.Drive(**{**d.__dict__, "augmented": False}), xi, np.zeros(n),
                                        np.zeros(n), D)
    assert np.allclose(dphi2, d.strength * inten, rtol=0, atol=1e-14)


def test_oracle_conserves_energy_and_mass():
    """Physics pin independent of the reference's vectors: along an RK4
    trajectory of a water wave the oracle's kinetic + potential energy
    (Energies.cuh:136-204) and mass drift only at the integrator's order.
    Halving dt shrinks the energy drift by more than 2^4."""
    from superfluid_dynamics_gb300 import workloads as W
    s = W.random_modes(64, seed=2)
    P = O.Problem()

    def invariants(x, y, phi):
        (dx, dy, _), _ = O.rhs(P, x, y, phi)
        return O.invariants(P, x, y, phi, dx, dy)

    i0 = invariants(s.x, s.y, s.phi)
    drift = []
    for steps, dt in ((200, 0.005), (400, 0.0025)):
        (x, y, p), _ = O.rk4_steps(P, s.x, s.y, s.phi, dt, steps)
        i1 = invariants(x, y, p)
        drift.append(abs((i1[0] + i1[1]) - (i0[0] + i0[1])) / abs(i0[0] + i0[1]))
        assert abs(i1[4] - i0[4]) < 1e-14
    assert drift[0] < 1e-11 and drift[0] / drift[1] > 16.0, drift


# --- the reference's own FP64 CUDA path (oracle/ref_harness.cu)
REF_CASES = ["ref_helium_n128_h10", "ref_helium_n128_h5", "ref_helium_n256_h8", "ref_water_n128_modes"]


@pytest.mark.parametrize("name", REF_CASES)
def test_oracle_matches_reference_cuda_path(name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    h = float(d["depth"])
    prob = O.Problem(physics=O.HELIUM, depth=h) if "helium" in name else O.Problem()
    (vx, vy, dphi, a, _, _), info = O.rhs(prob, d["x"], d["y"], d["phi"], diagnostics=True)
    assert rel(vx + 1j * vy, d["vx"] + 1j * d["vy"]) < 1e-12
    assert rel(dphi, d["dphi"]) < 1e-12
    assert rel(a, d["a"]) < 1e-12
