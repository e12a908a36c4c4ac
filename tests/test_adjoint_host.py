"""Host logic of the autograd wrapper (superfluid_dynamics_gb300.adjoint): the
engine keeps one recorded trajectory, so a backward must belong to the latest
forward of its Trajectory.  A stub engine (final = 2 state0, gradient 2 g)
stands in for the CUDA one."""
import numpy as np
import pytest
import torch

from superfluid_dynamics_gb300 import adjoint


class _StubEngine:
    def rk4_record(self, dt, steps, every, state0):
        return 2.0 * state0

    def rk4_vjp(self, g):
        return 2.0 * g, float(g.sum())


def _traj():
    t = adjoint.Trajectory.__new__(adjoint.Trajectory)
    t.dt, t.steps, t.checkpoint_every = 1e-3, 4, 2
    t.engine = _StubEngine()
    t._recordings = 0
    t._apply_param = lambda value: None
    return t


def test_backward_of_latest_forward():
    t = _traj()
    s0 = torch.arange(6, dtype=torch.float64, requires_grad=True)
    p = torch.tensor(1.5, dtype=torch.float64, requires_grad=True)
    t(s0, p).sum().backward()
    assert torch.equal(s0.grad, torch.full((6,), 2.0, dtype=torch.float64)) and p.grad.item() == 6.0


def test_backward_after_a_newer_forward_raises():
    t = _traj()
    s0 = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    p = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    first = t(s0, p)
    second = t(s0, p)
    with pytest.raises(RuntimeError, match="re-recorded"):
        first.sum().backward()
    second.sum().backward()
    assert np.array_equal(s0.grad.numpy(), np.full(6, 2.0))
