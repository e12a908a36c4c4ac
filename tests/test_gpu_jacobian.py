"""GPU tests of the RHS Jacobian: the reference's central-difference export
calculateJacobian (batched FP64 engine) against central differences of the
FP64 CPU oracle, and the exact adjoint Jacobian against the export.
Tolerances: export vs oracle FD 1e-6 of max |J| (both FD with the same
epsilon; their difference is RHS round-off / epsilon); exact vs FD 1e-5 of
max |J| (FD truncation, epsilon = 1e-6)."""
import numpy as np
import pytest

from oracle import oracle as O
import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

L, RHO, KAPPA, DEPTH = 1e-6, 150.0, 0.0, 15e-9   # SI, the reference's film studies


def nondim_depth():
    return DEPTH / (L / (2 * np.pi))


def film_state(n, seed=12):
    rng = np.random.default_rng(seed)
    xi = W.nodes(n)
    h = nondim_depth()
    y = 0.05 * h * np.cos(xi + rng.uniform(0, 6.28)) + 0.02 * h * np.sin(3 * xi)
    phi = 1e-3 * np.sin(2 * xi)
    return xi, y, phi


def test_jacobian_export_matches_oracle_fd():
    n, eps = 32, 1e-6
    x, y, phi = film_state(n)
    rc, J = sfd.SimulationManager().calculate_jacobian(x, y, phi, L, RHO, KAPPA, DEPTH, eps)
    assert rc == 0 and J.shape == (3 * n, 3 * n)
    P = O.Problem(physics=sfd.HELIUM, depth=nondim_depth(), rho=RHO / 150.0)
    s = np.concatenate([x, y, phi])
    Jo = np.empty_like(J)
    for c in range(3 * n):
        sp, sm = s.copy(), s.copy()
        sp[c] += eps
        sm[c] -= eps
        fp = np.concatenate(O.rhs(P, sp[:n], sp[n:2 * n], sp[2 * n:])[0])
        fm = np.concatenate(O.rhs(P, sm[:n], sm[n:2 * n], sm[2 * n:])[0])
        Jo[:, c] = (fp - fm) / (2 * eps)
    assert np.abs(J - Jo).max() <= 1e-6 * np.abs(Jo).max(), np.abs(J - Jo).max() / np.abs(Jo).max()


def test_exact_jacobian_matches_fd_export():
    n = 64
    x, y, phi = film_state(n, seed=13)
    rc, Jfd = sfd.SimulationManager().calculate_jacobian(x, y, phi, L, RHO, KAPPA, DEPTH, 1e-6)
    assert rc == 0
    phys = sfd.HeliumBoundaryProblem(depth=nondim_depth())
    with sfd.Engine(n, phys, sfd.Options(precision=sfd.PRECISION_FP64, use_graphs=False)) as e:
        Jx = e.jacobian(np.concatenate([x, y, phi]))
    assert np.abs(Jx - Jfd).max() <= 1e-5 * np.abs(Jx).max(), np.abs(Jx - Jfd).max() / np.abs(Jx).max()
    # the phi -> dphi block is not identically zero and the x -> dx block is not the identity
    assert np.abs(Jx[2 * n:, 2 * n:]).max() > 0
