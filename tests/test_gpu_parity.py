"""GPU parity: the CUDA engine (through the C ABI) against the FP64 oracle on
the same seeded inputs, the reference NumPy golden fixtures and the re-derived
known-answer tests.  Tolerances:
  FP64 mode  : max |diff| <= 1e-11 * max |oracle|   (RHS; FFT / summation order only)
  mixed mode : max |diff| <= 1e-10 * max |oracle|   (refined to ~1e-12 in practice)
  trajectories: 1e-9 relative after the stated steps
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
PREC = {"fp64": sfd.PRECISION_FP64, "mixed": sfd.PRECISION_MIXED}
TOL = {"fp64": 1e-11, "mixed": 1e-10}


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def oracle_problem(p: sfd.Physics) -> O.Problem:
    return O.Problem(physics=p.physics, rho=p.rho, depth=p.depth, A3=p.A3, gravity=p.gravity, U=p.U,
                     infinite_depth=p.infinite_depth)


def engine_rhs(n, phys, x, y, phi, prec, **kw):
    with sfd.Engine(n, phys, sfd.Options(precision=PREC[prec], **kw)) as e:
        e.set_state(x, y, phi)
        out = e.rhs(diagnostics=True)
        st = e.status()
    return out, st


def check_rhs(n, phys, s, prec, tol=None):
    (dx, dy, dphi, a, zp, zpp), st = engine_rhs(n, phys, s.x, s.y, s.phi, prec)
    (ox, oy, op, oa, ozp, ozpp), info = O.rhs(oracle_problem(phys), s.x, s.y, s.phi, diagnostics=True)
    tol = tol or TOL[prec]
    assert rel(dx + 1j * dy, ox + 1j * oy) < tol
    assert rel(dphi, op) < tol or np.abs(dphi - op).max() < tol * max(np.abs(ox).max(), 1e-300)
    assert rel(a, oa) < tol
    assert rel(zp, ozp) < 1e-13 and rel(zpp, ozpp) < 1e-11
    assert (st[0] & (sfd._lib.STATUS_NONFINITE | sfd._lib.STATUS_ZERO_PIVOT)).max() == 0


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("n", [4, 8, 32, 96, 128, 160, 1024])
def test_water_rhs(prec, n):
    check_rhs(n, sfd.WaterBoundaryProblem(), W.random_modes(n, seed=2), prec)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_water_steep_rhs(prec):
    check_rhs(256, sfd.WaterBoundaryProblem(), W.linear_wave(256, 0.3), prec)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("n,h,A3", [(64, 10.0, None), (96, 5.0, 800.0), (224, 12.0, 1500.0), (512, 10.0, 1e3)])
def test_helium_rhs(prec, n, h, A3):
    xi = W.nodes(n)
    s = W.Surface(xi.copy(), 0.05 * h * np.cos(3 * xi), 0.01 * np.sin(2 * xi))
    check_rhs(n, sfd.HeliumBoundaryProblem(h, A3), s, prec)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_helium_infinite_depth_and_water_rho(prec):
    s = W.random_modes(128, seed=5)
    check_rhs(128, sfd.HeliumBoundaryProblem(3.0, infinite_depth=True), s, prec)
    check_rhs(128, sfd.WaterBoundaryProblem(rho=0.3), s, prec)


@pytest.mark.parametrize("name", ["o1_linear_wave_n128_rhs", "o1_modes_seed2_n64_rhs", "o1_modes_seed2_n256_rhs",
                                  "o1_steep_n64_rhs"])
def test_golden_reference_numpy(name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    n = d["x"].size
    (dx, dy, dphi, a, zp, zpp), _ = engine_rhs(n, sfd.WaterBoundaryProblem(), d["x"], d["y"], d["phi"], "fp64")
    assert rel(dx + 1j * dy, d["vx"] + 1j * d["vy"]) < 1e-11
    assert rel(dphi, d["dphi"]) < 1e-11
    assert rel(a, d["a"]) < 1e-11


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["ref_helium_n128_h10", "ref_helium_n128_h5", "ref_helium_n256_h8",
                                  "ref_water_n128_modes"])
def test_golden_reference_cuda_path(name, prec):
    """The engine against outputs of the reference's own FP64 CUDA path
    (tests/golden/make_ref_fixtures.py): helium with A3 = h^4/3, and water."""
    d = np.load(os.path.join(GOLD, name + ".npz"))
    n, h = d["x"].size, float(d["depth"])
    phys = sfd.HeliumBoundaryProblem(h) if "helium" in name else sfd.WaterBoundaryProblem()
    (dx, dy, dphi, a, zp, zpp), _ = engine_rhs(n, phys, d["x"], d["y"], d["phi"], prec)
    assert rel(dx + 1j * dy, d["vx"] + 1j * d["vy"]) < TOL[prec]
    assert rel(dphi, d["dphi"]) < TOL[prec]
    assert rel(a, d["a"]) < TOL[prec]


def stokes(N, h, omega, t):
    j = 2 * np.pi * np.arange(N) / N
    X = j - h * np.sin(j - omega * t)
    Y = h * np.cos(j - omega * t)
    Phi = h * omega * np.sin(j - omega * t)
    s1, s2 = 2 * np.pi / N, 4 * np.pi ** 2 / N ** 2
    Zp = s1 * ((1 - h * np.cos(j - omega * t)) + 1j * (-h * np.sin(j - omega * t)))
    Zpp = s2 * ((h * np.sin(j - omega * t)) + 1j * (-h * np.cos(j - omega * t)))
    return X, Y, Phi, Zp, Zpp


def test_stokes_derivatives_known_answer():
    # MatrixMTests.cuh:477-607: z', z'' of a Lagrangian Stokes wave at N=1024, 1e-14
    X, Y, Phi, Zp, Zpp = stokes(1024, 0.5, 10.0, 0.0)
    (dx, dy, dphi, a, zp, zpp), _ = engine_rhs(1024, sfd.WaterBoundaryProblem(), X, Y, Phi, "fp64")
    assert np.abs(zp - Zp).max() < 1e-14
    assert np.abs(zpp - Zpp).max() < 1e-14


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_rk4_trajectory_water(prec):
    d = np.load(os.path.join(GOLD, "o1_linear_wave_n128_rk4.npz"))
    with sfd.Engine(128, sfd.WaterBoundaryProblem(), sfd.Options(precision=PREC[prec])) as e:
        e.set_state(d["x"], d["y"], d["phi"])
        e.step(0.01, 10)
        x, y, phi = e.get_state()
        assert np.abs(x - d["x_10"]).max() < 1e-11 and np.abs(y - d["y_10"]).max() < 1e-11
        e.step(0.01, 90)
        x, y, phi = e.get_state()
    scale = np.abs(d["x_100"]).max()
    assert np.abs(x - d["x_100"]).max() / scale < 1e-10
    assert np.abs(y - d["y_100"]).max() / scale < 1e-10
    assert np.abs(phi - d["phi_100"]).max() / scale < 1e-10


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_rk4_trajectory_helium(prec):
    n, h = 96, 8.0
    xi = W.nodes(n)
    x0, y0, p0 = xi.copy(), 0.3 * np.cos(2 * xi), np.zeros(n)
    with sfd.Engine(n, sfd.HeliumBoundaryProblem(h, 900.0), sfd.Options(precision=PREC[prec])) as e:
        e.set_state(x0, y0, p0)
        e.step(1e-3, 20)
        x, y, phi = e.get_state()
    (rx, ry, rp), info = O.rk4_steps(O.Problem(physics=O.HELIUM, depth=h, A3=900.0), x0, y0, p0, 1e-3, 20)
    assert max(np.abs(x - rx).max(), np.abs(y - ry).max(), np.abs(phi - rp).max()) < 1e-10


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_uneven_helium_batch(prec):
    surfs = W.helium_batch(6, seed=3, n_max=384)
    phys = [sfd.HeliumBoundaryProblem(s.depth, s.A3) for s in surfs]
    with sfd.Engine([s.n for s in surfs], phys, sfd.Options(precision=PREC[prec])) as e:
        e.set_state(np.concatenate([s.x for s in surfs]), np.concatenate([s.y for s in surfs]),
                    np.concatenate([s.phi for s in surfs]))
        dx, dy, dphi = e.rhs()
        parts = [e.split(v) for v in (dx, dy, dphi)]
    for i, s in enumerate(surfs):
        (ox, oy, op), info = O.rhs(O.Problem(physics=O.HELIUM, depth=s.depth, A3=s.A3), s.x, s.y, s.phi)
        scale = max(np.abs(ox).max(), np.abs(oy).max(), np.abs(op).max())
        err = max(np.abs(parts[0][i] - ox).max(), np.abs(parts[1][i] - oy).max(), np.abs(parts[2][i] - op).max())
        assert err < TOL[prec] * scale, (i, s.n, err / scale)


def test_invariants_match_oracle():
    s = W.random_modes(256, seed=2)
    with sfd.Engine(256, sfd.WaterBoundaryProblem(), sfd.Options(precision=sfd.PRECISION_FP64)) as e:
        e.set_state(s.x, s.y, s.phi)
        inv = e.invariants(kappa=0.5)[0]
        dx, dy, dphi = e.rhs()
    ref = O.invariants(O.Problem(), s.x, s.y, s.phi, dx, dy, kappa=0.5)
    assert np.abs(inv - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


# --------------------------------------------------------------- reference-compatible exports
def nondim(L, rho, kappa, depth):
    bl = L / (2 * np.pi)
    ba = 3 * 3.5e-24 / depth ** 4
    return depth / bl


def test_calculate_rhs_from_vectors_matches_oracle():
    L, depth = 1e-3, 2e-8
    h = nondim(L, 145.0, 0.0, depth)
    n = 128
    xi = W.nodes(n)
    x, y, phi = xi.copy(), 0.02 * h * np.cos(xi), 0.001 * np.sin(xi)
    sm = sfd.SimulationManager()
    rc, vx, vy, dphi = sm.calculate_rhs_from_vectors(x, y, phi, L, 145.0, 0.0, depth)
    assert rc == 0
    (ox, oy, op), info = O.rhs(O.Problem(physics=O.HELIUM, depth=h), x, y, phi)
    assert rel(vx + 1j * vy, ox + 1j * oy) < 1e-11 and rel(dphi, op) < 1e-9
    rc2, vx2, vy2, dphi2 = sm.calculate_rhs256_from_vectors_batched(np.tile(W.nodes(256), 3),
                                                                    np.tile(0.02 * h * np.cos(W.nodes(256)), 3),
                                                                    np.tile(np.zeros(256), 3), L, 145.0, 0.0,
                                                                    depth, 3)
    assert rc2 == 0 and np.allclose(vx2[:256], vx2[256:512], atol=0, rtol=0)


def test_vorticities_and_fft_exports():
    L, depth = 1e-3, 2e-8
    h = nondim(L, 145.0, 0.0, depth)
    n = 256
    xi = W.nodes(n)
    Z = xi + 1j * (0.02 * h * np.cos(2 * xi))
    phi = (0.001 * np.sin(2 * xi)).astype(complex)
    sm = sfd.SimulationManager()
    rc, a, Zp, Zpp = sm.calculate_vorticities256_from_vectors(Z, phi, L, 145.0, 0.0, depth)
    assert rc == 0
    (_, _, _, oa, ozp, ozpp), _ = O.rhs(O.Problem(physics=O.HELIUM, depth=h), Z.real, Z.imag, phi.real,
                                        diagnostics=True)
    assert rel(a, oa) < 1e-11 and rel(Zp, ozp) < 1e-13
    sig = np.exp(1j * 3 * xi) + 0.5 * np.sin(5 * xi)
    rc, out = sm.calculate_derivativeFFT256(sig)
    assert rc == 0
    assert rel(out, O.fft_derivative(sig)) < 1e-13


def test_rhs256_from_file_export(tmp_path):
    """calculateRHS256FromFile (Export.cu:42-113): the state file's y is scaled
    by 2 pi / L, the RHS is the 256-node helium RHS of the vector export, and
    the output state file carries (dx, dy), dphi and the nondimensional
    properties with initial_amplitude = (max y - min y) / 2 and rhs = true."""
    from superfluid_dynamics_gb300 import h5io
    L, depth = 1e-3, 2e-8
    h = nondim(L, 145.0, 0.0, depth)
    n = 256
    xi = W.nodes(n)
    scale = 2 * np.pi / L
    y_file = (0.02 * h * np.cos(2 * xi)) / scale
    phi = 0.001 * np.sin(2 * xi)
    src, out = str(tmp_path / "state.h5"), str(tmp_path / "rhs.h5")
    h5io.save_state_file(src, xi + 1j * y_file, phi, {"depth": depth})
    sm = sfd.SimulationManager()
    assert sm.calculate_rhs256(src, out, L, 145.0, 0.0, depth) == 0
    y = scale * y_file
    rc, vx, vy, dphi = sm.calculate_rhs256_from_vectors(xi, y, phi, L, 145.0, 0.0, depth)
    assert rc == 0
    ds, attrs = h5io.read(out)
    itf, pot = ds["interface"], ds["potential"]
    assert itf.shape == (n, 2) and pot.shape == (n,)
    assert rel(itf[:, 0] + 1j * itf[:, 1], vx + 1j * vy) < 1e-13 and rel(pot, dphi) < 1e-13
    (ox, oy, op), _ = O.rhs(O.Problem(physics=O.HELIUM, depth=h), xi, y, phi)
    assert rel(itf[:, 0] + 1j * itf[:, 1], ox + 1j * oy) < 1e-11 and rel(pot, op) < 1e-9
    assert attrs["rhs"] is True and attrs["U"] == 0.0 and attrs["kappa"] == 0.0
    assert attrs["initial_amplitude"] == (y.max() - y.min()) / 2.0
    assert np.isclose(attrs["depth"], h, rtol=1e-14, atol=0) and np.isclose(attrs["rho"], 145.0 / 150.0, rtol=1e-15, atol=0)


def test_integrate_simulation_rk4_export():
    L, depth = 1e-3, 2e-8
    n = 64
    h = nondim(L, 145.0, 0.0, depth)
    xi = W.nodes(n)
    x, y, phi = xi.copy(), 0.05 * h * np.cos(xi), np.zeros(n)
    # SI times: base_time = sqrt(bl / (3 alpha / d^4))
    bl = L / (2 * np.pi)
    bt = np.sqrt(bl / (3 * 3.5e-24 / depth ** 4))
    sm = sfd.SimulationManager()
    S, T = sm.integrate_simulation_rk4(x, y, phi, L, 145.0, 0.0, depth, 0.0, 5e-3 * bt * 4 + 1e-6 * bt,
                                       5e-3 * bt, True)
    assert S.shape == (5, 3 * n) and T.shape == (5,)
    (rx, ry, rp), _ = O.rk4_steps(O.Problem(physics=O.HELIUM, depth=h), x, y, phi, 5e-3, 4)
    assert np.abs(S[-1, :n] - rx).max() < 1e-11 and np.abs(S[-1, n:2 * n] - ry).max() < 1e-11
    assert np.abs(S[0, :n] - x).max() == 0


def test_errors_are_reported_not_fatal():
    with pytest.raises(sfd.SfdError):
        sfd.Engine(9000, sfd.WaterBoundaryProblem())
    with pytest.raises(sfd.SfdError):
        sfd.Engine(64, sfd.HeliumBoundaryProblem(-1.0))
    sm = sfd.SimulationManager()
    rc, *_ = sm.calculate_rhs_from_vectors(np.zeros(9000), np.zeros(9000), np.zeros(9000), 1e-3, 145.0, 0.0, 2e-8)
    assert rc == -1


def test_nonfinite_state_sets_status():
    s = W.random_modes(64, seed=2)
    y = s.y.copy()
    y[5] = np.nan
    with sfd.Engine(64, sfd.WaterBoundaryProblem(), sfd.Options(precision=sfd.PRECISION_FP64)) as e:
        e.set_state(s.x, y, s.phi)
        e.rhs()
        st, _, _ = e.status()
    assert st[0] & sfd._lib.STATUS_NONFINITE


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_mixing_cluster_and_single_cta_transforms(prec):
    # n % 64 == 0 and n >= 512 use the cluster-distributed transforms; others one CTA
    sizes = [512, 96, 640, 1152, 160, 1024, 2048]
    surfs = []
    for i, n in enumerate(sizes):
        xi = W.nodes(n)
        surfs.append(W.Surface(xi.copy(), 0.04 * np.cos((i + 1) * xi) + 0.01 * np.sin(3 * xi),
                               0.02 * np.sin((i + 1) * xi)))
    with sfd.Engine(sizes, sfd.WaterBoundaryProblem(), sfd.Options(precision=PREC[prec])) as e:
        e.set_state(np.concatenate([s.x for s in surfs]), np.concatenate([s.y for s in surfs]),
                    np.concatenate([s.phi for s in surfs]))
        dx, dy, dphi, a, zp, zpp = e.rhs(diagnostics=True)
        parts = [e.split(v) for v in (dx, dy, dphi, zp, zpp)]
    for i, s in enumerate(surfs):
        (ox, oy, op, oa, ozp, ozpp), _ = O.rhs(O.Problem(), s.x, s.y, s.phi, diagnostics=True)
        assert rel(parts[3][i], ozp) < 1e-13 and rel(parts[4][i], ozpp) < 1e-11
        assert rel(parts[0][i] + 1j * parts[1][i], ox + 1j * oy) < TOL[prec]
        assert rel(parts[2][i], op) < TOL[prec]


@pytest.mark.parametrize("n", [256, 640, 1024, 3072])
def test_tensor_core_preconditioner(n):
    # The tcgen05 (3 x bf16-split) Gauss-Jordan update must give a usable inverse on
    # its own (no refinement: a = X phi' to ~1e-4), and the refined result must match.
    # n = 3072: four tiles per CTA of the update, so its stage ring and both tensor-memory
    # accumulators are reused.
    s = W.random_modes(n, seed=11)
    (ox, oy, op, oa, _, _), _ = O.rhs(O.Problem(), s.x, s.y, s.phi, diagnostics=True)
    for tc in (True, False):
        out0, st0 = engine_rhs(n, sfd.WaterBoundaryProblem(), s.x, s.y, s.phi, "mixed", refine_iters=0,
                               tensor_cores=tc)
        assert rel(out0[3], oa) < (1e-3 if tc else 1e-5)
        out3, st3 = engine_rhs(n, sfd.WaterBoundaryProblem(), s.x, s.y, s.phi, "mixed", refine_iters=3,
                               tensor_cores=tc)
        assert rel(out3[3], oa) < 1e-10
        assert rel(out3[0] + 1j * out3[1], ox + 1j * oy) < 1e-10
        assert (st3[0] & (sfd._lib.STATUS_TIMEOUT | sfd._lib.STATUS_NONFINITE)).max() == 0


def test_autotuned_sum_shape_is_valid_and_parity_holds():
    """The boundary-sum autotuner (first step of an engine) picks 2, 4 or 8
    source groups per CTA; the stepped result still matches the oracle."""
    n, dt, steps = 256, 0.005, 3
    s = W.random_modes(n, seed=2)
    with sfd.Engine(n, sfd.WaterBoundaryProblem(), sfd.Options(precision=sfd.PRECISION_MIXED)) as e:
        e.set_state(s.x, s.y, s.phi)
        e.step(dt, steps)
        t = e.tuning()
        gx, gy, gp = e.get_state()
    assert t["fp32"] in (2, 4, 8) and t["df"] in (2, 4, 8)
    (ox, oy, op), _ = O.rk4_steps(O.Problem(), s.x, s.y, s.phi, dt, steps)
    assert rel(gx + 1j * gy, ox + 1j * oy) < 1e-9 and rel(gp, op) < 1e-9
