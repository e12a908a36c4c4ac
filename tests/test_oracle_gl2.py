"""The oracle's two-stage Gauss-Legendre (the reference's GaussLegendre2,
GaussLegendre.cuh:216-605) pinned by known answers: one step on y' = lam y is
the (2,2) Pade approximant of exp(h lam); the global error on a rotation is
fourth order; on the boundary problem it agrees with a fine RK4 run; a Newton
iteration cap of zero fails every halving and raises."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("lam", [-1.0, -3.0, -50.0, 2.0])
def test_gl2_step_is_the_pade_approximant(lam):
    h = 0.1
    ok, yn, _, _ = O.gl2_step(lambda y: lam * y, lambda y: np.array([[lam]]), np.array([1.0]), h)
    z = lam * h
    pade = (1 + z / 2 + z * z / 12) / (1 - z / 2 + z * z / 12)
    assert ok and abs(yn[0] - pade) <= 1e-14 * abs(pade)


def test_gl2_is_fourth_order_on_a_rotation():
    A = np.array([[0.0, 1.0], [-1.0, 0.0]])
    errs = []
    for h in (0.2, 0.1, 0.05):
        _, s = O.gl2_evolve(lambda y: A @ y, [1.0, 0.0], 0.0, 2.0, h, jac=lambda y: A)
        errs.append(np.abs(s[-1] - [np.cos(2.0), -np.sin(2.0)]).max())
    for a, b in zip(errs, errs[1:]):
        assert 14.0 < a / b < 18.0


def test_gl2_is_stable_on_a_stiff_linear_problem():
    lam = -1e4  # h lam = -1000: explicit RK4 would blow up
    _, s = O.gl2_evolve(lambda y: lam * y, [1.0], 0.0, 1.0, 0.1, jac=lambda y: np.array([[lam]]))
    assert np.all(np.abs(s[:, 0]) <= 1.0)


@pytest.mark.parametrize("case", ["water", "helium"])
def test_gl2_boundary_agrees_with_fine_rk4(case):
    n = 16
    xi = 2 * np.pi * np.arange(n) / n
    if case == "water":
        prob, amp = O.Problem(), 0.05
    else:
        prob, amp = O.Problem(physics=O.HELIUM, depth=10.0, A3=1e3), 0.5
    y0 = np.concatenate([xi, amp * np.cos(xi), 0.3 * amp * np.sin(xi)])
    t, s = O.gl2_evolve(O.boundary_rhs(prob), y0, 0.0, 0.03, 0.01)
    assert len(t) == 4
    (x, y, p), _ = O.rk4_steps(prob, y0[:n], y0[n:2 * n], y0[2 * n:], 0.001, 30)
    ref = np.concatenate([x, y, p])
    assert np.abs(s[-1] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_gl2_without_newton_iterations_fails():
    with pytest.raises(RuntimeError):
        O.gl2_evolve(lambda y: -y, [1.0], 0.0, 1.0, 0.1, jac=lambda y: np.array([[-1.0]]), max_newton=0,
                     max_halvings=2)
