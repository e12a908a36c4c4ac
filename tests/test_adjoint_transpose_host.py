"""Host check of the mathematics behind the mixed engines' transposed solve.

The reverse sweep of a mixed engine never forms M: it evaluates M^T lambda
matrix-free from the node data, with w = e^{iz} and p = w e^{-h},
    gC = i c1 conj(z') lambda,   gD = -i cI lambda,   b = w conj(gC),
    Sb_j = sum_{k != j} b_k / (w_j - w_k),   Tb_j = sum_k gD_k / (1 - p_j conj p_k),
    (M^T lambda)_j = Mdiag_j lambda_j + Re(i (sum gC - gC_j) + 2 i conj(Sb_j))
                     + Re(-i sum gD + 2 i Tb_j),
and it stores the pair matrices once per stage using R_kj = -R_jk and
I_kj = conj(I_jk).  Here that restatement (numpy) is compared with the
oracle's dense M (createM.cuh:43-92 as the oracle restates it) transposed,
for water and finite-depth helium surfaces; no GPU is involved.
"""
import numpy as np
import pytest

from oracle import oracle as O
from superfluid_dynamics_gb300 import workloads as W


def mt_lambda(Z, Zp, Zpp, lam, depth=None):
    """M^T lambda by the reverse sweep's formula (depth None: no image)."""
    c1 = 0.25 / np.pi
    image = depth is not None
    cI = c1 if image else 0.0
    w = np.exp(1j * Z)
    mdiag = 0.5 + c1 * np.imag(Zpp / Zp)
    gC = 1j * c1 * np.conj(Zp) * lam
    b = w * np.conj(gC)
    R = w[:, None] - w[None, :]          # w_j - w_k, row j
    np.fill_diagonal(R, 1.0)
    R = 1.0 / R
    np.fill_diagonal(R, 0.0)
    Sb = R @ b
    out = mdiag * lam + np.real(1j * (gC.sum() - gC) + 2j * np.conj(Sb))
    if image:
        p = w * np.exp(-depth)
        gD = -1j * cI * lam
        I = 1.0 / (1.0 - p[:, None] * np.conj(p[None, :]))
        out += np.real(-1j * gD.sum() + 2j * (I @ gD))
    return out, R, (I if image else None)


def surface_data(s):
    Z = s.x + 1j * s.y
    Zp, _, Zpp = O.zphi_derivative(Z, s.phi + 0j)
    return Z, Zp, Zpp


@pytest.mark.parametrize("case", ["water", "helium_h10", "helium_h2"])
@pytest.mark.parametrize("n", [32, 96])
def test_matrix_free_transpose_matches_dense(case, n):
    if case == "water":
        s = W.random_modes(n, seed=2)
        prob, depth = O.Problem(), None
    else:
        h = 10.0 if case == "helium_h10" else 2.0
        s = W.random_modes(n, seed=5)
        s.y *= 0.02 * h / max(np.abs(s.y).max(), 1e-300)   # a film: amplitude 2 % of the depth
        prob, depth = O.Problem(physics=1, depth=h, A3=1e3), h
    Z, Zp, Zpp = surface_data(s)
    M = O.create_M(prob, Z, Zp, Zpp)
    lam = np.random.default_rng(3).standard_normal(n)
    got, R, I = mt_lambda(Z, Zp, Zpp, lam, depth)
    ref = M.T @ lam
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), np.abs(got - ref).max() / np.abs(ref).max()
    # the symmetries the pair-reciprocal kernel stores with: R exactly (a
    # negated difference has the negated reciprocal), I to rounding (the two
    # products p_j conj p_k and p_k conj p_j round separately)
    assert np.array_equal(R.T, -R)
    if I is not None:
        assert np.abs(I.T - np.conj(I)).max() <= 1e-15 * np.abs(I).max()


def test_transposed_refinement_converges_with_an_inexact_inverse():
    """lambda = X^T g, then lambda += X^T (g - M^T lambda): with X an inverse of
    M perturbed by 1e-4 (as a stale or reduced-precision preconditioner is),
    three corrections reach the FP64 level."""
    n = 64
    s = W.random_modes(n, seed=2)
    Z, Zp, Zpp = surface_data(s)
    M = O.create_M(O.Problem(), Z, Zp, Zpp)
    rng = np.random.default_rng(4)
    X = np.linalg.inv(M) * (1.0 + 1e-4 * rng.standard_normal((n, n)))
    g = rng.standard_normal(n)
    lam = X.T @ g
    for _ in range(3):
        r = g - mt_lambda(Z, Zp, Zpp, lam)[0]
        lam = lam + X.T @ r
    r = g - M.T @ lam
    assert np.abs(r).max() <= 1e-13 * np.abs(g).max()
