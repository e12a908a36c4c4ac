"""Argument errors of the engine API on a live device: refused with an error
code and a message, before any work or copy, leaving the engine usable."""
import numpy as np
import pytest

import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_step_host_rejects_bad_arguments_and_leaves_arrays():
    """A non-finite time step or a negative step count is refused before any
    copy; the host arrays are left as they were and the engine stays usable."""
    n = 256
    s = W.random_modes(n, seed=3)
    with sfd.Engine(n, sfd.WaterBoundaryProblem(), sfd.Options(autotune=False)) as e:
        x, y, p = s.x.copy(), s.y.copy(), s.phi.copy()
        for dt, steps in ((float("nan"), 1), (float("inf"), 1), (0.005, -1)):
            with pytest.raises(sfd.SfdError):
                e.step_host(x, y, p, dt, steps)
            assert np.array_equal(x, s.x) and np.array_equal(y, s.y) and np.array_equal(p, s.phi)
        with pytest.raises(sfd.SfdError, match="finite"):
            e.step(float("nan"), 1)
        e.step_host(x, y, p, 0.005, 1)
        assert np.all(np.isfinite(x)) and not np.array_equal(y, s.y)


@pytest.mark.parametrize("opts, msg", [(sfd.Options(precision=7), "unknown precision 7"),
                                       (sfd.Options(device=4096), "device 4096 out of range")])
def test_create_rejects_bad_options(opts, msg):
    with pytest.raises(sfd.SfdError, match=msg):
        sfd.Engine(128, sfd.WaterBoundaryProblem(), opts)
    # the failed creation leaves nothing behind: the next engine works
    with sfd.Engine(128, sfd.WaterBoundaryProblem(), sfd.Options(autotune=False)) as e:
        s = W.random_modes(128, seed=1)
        e.set_state(s.x, s.y, s.phi)
        e.step(0.005, 2)
        assert np.all(np.isfinite(np.concatenate(e.get_state())))


@pytest.mark.parametrize("kw, msg", [({"min_alpha": 0.0}, "min_alpha"), ({"min_alpha": float("nan")}, "min_alpha"),
                                     ({"armijo_c": 1.5}, "armijo_c"), ({"fd_eps": float("inf")}, "fd_eps"),
                                     ({"step": float("inf")}, "step"), ({"t1": float("inf")}, "finite")])
def test_gl2_rejects_options_that_cannot_end(kw, msg):
    """A line search with min_alpha <= 0 never ends on a non-finite trial, and
    an infinite end time never ends: both are refused up front."""
    n = 64
    s = W.random_modes(n, seed=4)
    t1 = kw.pop("t1", 0.05)
    with sfd.Engine(n, sfd.WaterBoundaryProblem(), sfd.Options(precision=sfd.PRECISION_FP64)) as e:
        e.set_state(s.x, s.y, s.phi)
        with pytest.raises(sfd.SfdError, match=msg):
            e.evolve_gl2(0.0, t1, **kw)
        res, times = e.evolve_gl2(0.0, 0.02, step=0.01)
        assert res["steps"] == 2 and np.allclose(times, [0.01, 0.02])


def test_rkf45_rejects_infinite_end_time():
    n = 64
    s = W.random_modes(n, seed=4)
    with sfd.Engine(n, sfd.WaterBoundaryProblem(), sfd.Options(precision=sfd.PRECISION_FP64)) as e:
        e.set_state(s.x, s.y, s.phi)
        with pytest.raises(sfd.SfdError, match="finite"):
            e.evolve_rkf45(0.0, float("inf"))
        with pytest.raises(sfd.SfdError, match="h0"):
            e.evolve_rkf45(0.0, 0.1, h0=float("nan"))
