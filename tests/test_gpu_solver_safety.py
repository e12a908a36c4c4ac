"""Solver safety on the GPU, checked against the oracle.

* The dense solver behind MatrixSolver::solve (sfd_dense_solve) factors with
  partial pivoting, as cusolverDnDgetrf does (MatrixSolver.cuh:123-125): a
  matrix that needs row exchanges is solved to oracle accuracy (the oracle's
  LU pivots the same way) and the exchange is reported.
* The engine's solve checks its final residual against refine_tol and runs
  gated extra corrections where it is above: forced on (a tolerance below
  round-off) the FP64 refinement runs, reports the stall and still matches
  the oracle.
* A deliberately stale preconditioner (never rebuilt while a water wave
  evolves) is caught: without extra corrections the stall bit comes up and
  the host rebuilds the preconditioner; with them the residual is brought
  back under the tolerance.  Either way the trajectory stays on the FP64 one.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import _lib
from superfluid_dynamics_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    return torch


def _dense_solve(torch, mats, rhs):
    """sfd_dense_solve on `batch` row-major matrices (batch, n, n) and
    right-hand sides (batch, n); returns the solutions and status words."""
    L = _lib.load()
    batch, n, _ = mats.shape
    Mc = torch.tensor(np.concatenate([m.ravel(order="F") for m in mats]), dtype=torch.float64, device="cuda")
    b = torch.tensor(rhs.ravel(), dtype=torch.float64, device="cuda")
    x = torch.empty(batch * n, dtype=torch.float64, device="cuda")
    h = ctypes.c_void_p()
    assert L.sfd_dense_solver_create(n, batch, ctypes.byref(h)) == 0, L.sfd_last_error()
    try:
        st = (ctypes.c_uint * batch)()
        rc = L.sfd_dense_solve(h, ctypes.c_void_p(Mc.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                               ctypes.c_void_p(x.data_ptr()), st)
        assert rc == 0, L.sfd_last_error()
        torch.cuda.synchronize()
    finally:
        L.sfd_dense_solver_destroy(h)
    return x.cpu().numpy().reshape(batch, n), np.array(list(st), dtype=np.uint32)


def test_dense_solve_exchanges_rows_like_getrf():
    torch = _torch()
    # 2 x 2 permutation: no LU without an exchange exists
    x, st = _dense_solve(torch, np.array([[[0.0, 1.0], [1.0, 0.0]]]), np.array([[1.0, 2.0]]))
    assert np.array_equal(x[0], [2.0, 1.0])
    assert st[0] & _lib.STATUS_PIVOT_SWAP and not st[0] & _lib.STATUS_ZERO_PIVOT
    # batched, several blocks of 64: small diagonals force exchanges in every panel
    rng = np.random.default_rng(17)
    n, batch = 300, 3
    mats = rng.standard_normal((batch, n, n))
    for m in mats:
        m[np.arange(n), np.arange(n)] *= 1e-3
    rhs = rng.standard_normal((batch, n))
    x, st = _dense_solve(torch, mats, rhs)
    for i in range(batch):
        ref, info = O.lu_solve(mats[i], rhs[i])
        assert info == 0
        assert np.abs(x[i] - ref).max() <= 1e-11 * np.abs(ref).max()
        assert np.abs(mats[i] @ x[i] - rhs[i]).max() <= 1e-10 * np.abs(rhs[i]).max()
        assert st[i] & _lib.STATUS_PIVOT_SWAP
    # a diagonally dominant system needs no exchange and reports none
    d = rng.standard_normal((1, 200, 200)) + 400.0 * np.eye(200)
    x, st = _dense_solve(torch, d, rhs[:1, :200])
    ref, _ = O.lu_solve(d[0], rhs[0, :200])
    assert np.abs(x[0] - ref).max() <= 1e-13 * np.abs(ref).max() and st[0] == 0


def test_dense_solve_reports_a_singular_matrix():
    torch = _torch()
    m = np.ones((1, 70, 70))
    _, st = _dense_solve(torch, m, np.ones((1, 70)))
    assert st[0] & _lib.STATUS_ZERO_PIVOT


def _rhs(n, phys, s, **kw):
    with sfd.Engine(n, phys, sfd.Options(**kw)) as e:
        e.set_state(s.x, s.y, s.phi)
        out = e.rhs()
        st, _, rn = e.status()
        ref = e.refinement()
    return out, st, rn, ref


def test_fp64_refinement_runs_and_reports_when_the_tolerance_is_below_roundoff():
    n = 192
    s = W.random_modes(n, seed=4)
    (ox, oy, op), _ = O.rhs(O.Problem(), s.x, s.y, s.phi)
    scale = max(np.abs(ox).max(), np.abs(op).max())
    (dx, dy, dp), st, rn, ref = _rhs(n, sfd.WaterBoundaryProblem(), s, precision=sfd.PRECISION_FP64,
                                     extra_iters=3, refine_tol=1e-300)
    assert ref["extra_iters"][0] == 3
    assert st[0] & _lib.STATUS_REFINE_STALL
    assert max(np.abs(dx - ox).max(), np.abs(dy - oy).max(), np.abs(dp - op).max()) <= 1e-11 * scale
    # at the default tolerance no correction is needed and no stall is reported
    (dx, dy, dp), st, rn, ref = _rhs(n, sfd.WaterBoundaryProblem(), s, precision=sfd.PRECISION_FP64)
    assert ref["extra_iters"][0] == 0 and st[0] == 0
    assert ref["rel_residual"][0] <= 1e-12
    assert max(np.abs(dx - ox).max(), np.abs(dy - oy).max(), np.abs(dp - op).max()) <= 1e-11 * scale


def test_mixed_extra_corrections_reach_the_tolerance():
    """One regular FP32 correction leaves a residual above a tight tolerance;
    the gated extra corrections bring it under, and the RHS matches the oracle."""
    n = 512
    s = W.random_modes(n, seed=2)
    (ox, oy, op), _ = O.rhs(O.Problem(), s.x, s.y, s.phi)
    scale = max(np.abs(ox).max(), np.abs(op).max())
    (dx, dy, dp), st, rn, ref = _rhs(n, sfd.WaterBoundaryProblem(), s, precision=sfd.PRECISION_MIXED,
                                     pre_iters=0, refine_iters=0, extra_iters=4, refine_tol=1e-12)
    assert ref["extra_iters"][0] >= 1
    assert ref["rel_residual"][0] <= 1e-12 and not st[0] & _lib.STATUS_REFINE_STALL
    assert max(np.abs(dx - ox).max(), np.abs(dy - oy).max(), np.abs(dp - op).max()) <= 1e-10 * scale


def _chunked(opt, s, steps, chunk):
    """Step in calls of `chunk` steps (the host acts on a stall flag between
    calls); per call: status word, max relative residual, extra corrections."""
    rec = []
    with sfd.Engine(s.n, sfd.WaterBoundaryProblem(), opt) as e:
        e.set_state(s.x, s.y, s.phi)
        for _ in range(steps // chunk):
            e.clear_status()
            e.step(0.005, chunk)
            st, _, _ = e.status()
            r = e.refinement()
            rec.append((int(st[0]), float(r["rel_residual"][0]), int(r["extra_iters"][0]), r["stall_rebuilds"]))
        return rec, np.concatenate(e.get_state())


def test_stale_preconditioner_is_caught_and_recovered():
    """A water wave stepped with the benchmarked solver settings (2 FP32
    pre-iterations, 2 corrections) and a preconditioner that is never
    rebuilt on schedule, under a tolerance of 1e-12 that a fresh inverse
    meets (~4e-13) and an ageing one soon misses."""
    s = W.linear_wave(512, 0.1)
    steps, chunk = 200, 10
    with sfd.Engine(512, sfd.WaterBoundaryProblem(), sfd.Options(precision=sfd.PRECISION_FP64)) as e:
        e.set_state(s.x, s.y, s.phi)
        e.step(0.005, steps)
        fp64 = np.concatenate(e.get_state())
    base = dict(precision=sfd.PRECISION_MIXED, refactor_every=10 ** 6, pre_iters=2, refine_iters=2, refine_tol=1e-12,
                autotune=False)
    # no extra corrections: the stall bit comes up, the host rebuilds the
    # preconditioner in-step, and the residual is back under the tolerance
    rec, got = _chunked(sfd.Options(extra_iters=0, **base), s, steps, chunk)
    stalls = [i for i, c in enumerate(rec) if c[0] & _lib.STATUS_REFINE_STALL]
    assert stalls, rec
    assert rec[-1][3] >= 1, rec
    assert any(not c[0] & _lib.STATUS_REFINE_STALL for c in rec[stalls[0] + 1:]), rec
    assert np.abs(got - fp64).max() <= 1e-10 * np.abs(fp64).max()
    # with extra corrections the residual is held under the tolerance without a rebuild
    rec, got = _chunked(sfd.Options(extra_iters=4, **base), s, steps, chunk)
    assert sum(c[2] for c in rec) >= 1, rec
    assert not any(c[0] & _lib.STATUS_REFINE_STALL for c in rec), rec
    assert max(c[1] for c in rec) <= 1e-12
    assert np.abs(got - fp64).max() <= 1e-10 * np.abs(fp64).max()
