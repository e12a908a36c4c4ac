"""Reverse mode of RK4 trajectories as a torch.autograd.Function.

The backward pass calls the hand-written CUDA adjoint (sfd_rk4_vjp): each
checkpoint segment of the trajectory is recomputed once with every RK4 stage
recorded and reversed stage by stage.  With an FP64 engine the records include
the LU factors of M and the transposed solve uses them; with a mixed engine
(the production forward) the transposed solve is refinement preconditioned by
the transpose of the engine's approximate inverse.  The reference has no
reverse mode; it differentiates by finite differences
(Python/integration/jacobian_tests.py:10-150).

    traj = Trajectory(n=512, physics=HeliumBoundaryProblem(depth=10.0, A3=1e3),
                      dt=1e-3, steps=500, checkpoint_every=50)
    final = traj(state0, A3)            # state0: torch float64 [3n]; A3: 0-d tensor
    loss = 0.5 * ((final[n:2 * n] - y_target) ** 2).sum()
    loss.backward()                     # gradients of state0 and A3
"""
from __future__ import annotations

import dataclasses

import numpy as np
import torch

from ._lib import HELIUM, PRECISION_FP64, PRECISION_MIXED
from .engine import Engine, Options, Physics


class _RK4Trajectory(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state0, param, traj):
        traj._apply_param(float(param))
        final = traj.engine.rk4_record(traj.dt, traj.steps, traj.checkpoint_every,
                                       state0.detach().cpu().numpy())
        traj._recordings += 1
        ctx.traj = traj
        ctx.recording = traj._recordings  # the engine keeps only the latest recording
        ctx.param_device = param.device
        return torch.from_numpy(final).to(state0.device)

    @staticmethod
    def backward(ctx, grad_final):
        traj = ctx.traj
        if traj._recordings != ctx.recording:
            raise RuntimeError("the trajectory was re-recorded before backward: "
                               "call backward before the next forward of the same Trajectory")
        g0, gp = traj.engine.rk4_vjp(grad_final.detach().cpu().numpy())
        return (torch.from_numpy(g0).to(grad_final.device),
                torch.tensor(gp, dtype=torch.float64, device=ctx.param_device), None)


class Trajectory:
    """An engine for one surface plus the RK4 settings of the trajectory.

    precision=PRECISION_FP64 (default) records LU factors and reproduces the
    FP64 engine's steps bitwise; PRECISION_MIXED runs the forward on the
    mixed engine (captured step graphs, preconditioner rebuilt every
    `refactor_every` steps) and reverses it with the preconditioned transposed
    solve.  The differentiated parameter is A3 for helium films and g for
    water.  The engine holds one recording, so the backward of a forward must
    come before the next forward on the same object (an out-of-order backward
    raises)."""

    def __init__(self, n: int, physics: Physics, dt: float, steps: int, checkpoint_every: int = 50,
                 device: int = 0, precision: int = PRECISION_FP64, refactor_every: int = 50):
        self.n = int(n)
        self.physics = physics
        self.dt = float(dt)
        self.steps = int(steps)
        self.checkpoint_every = int(checkpoint_every)
        if precision == PRECISION_MIXED:
            opts = Options(precision=PRECISION_MIXED, pre_iters=2, refactor_every=int(refactor_every),
                           autotune=False, device=device)
        else:
            opts = Options(precision=PRECISION_FP64, use_graphs=False, device=device)
        self.engine = Engine(self.n, physics, opts)
        self._recordings = 0  # forwards so far; a backward must belong to the latest

    def _apply_param(self, value: float) -> None:
        fields = {f.name: getattr(self.physics, f.name) for f in dataclasses.fields(Physics)}
        fields["A3" if self.physics.physics == HELIUM else "gravity"] = value
        self.engine.set_problem(Physics(**fields))

    def __call__(self, state0: torch.Tensor, param: torch.Tensor) -> torch.Tensor:
        return _RK4Trajectory.apply(state0, param, self)

    def close(self) -> None:
        self.engine.close()


def fourier_basis(n: int, modes: int = 32) -> torch.Tensor:
    """[2 modes, n] basis: rows cos(m xi) for m = 1..modes, then sin(m xi)."""
    xi = 2 * np.pi * np.arange(n) / n
    m = np.arange(1, modes + 1)[:, None]
    return torch.from_numpy(np.concatenate([np.cos(m * xi), np.sin(m * xi)]))


def film_state(coeffs: torch.Tensor, basis: torch.Tensor) -> torch.Tensor:
    """[x | y | phi] with x = xi, y = coeffs @ basis, phi = 0 (differentiable in coeffs)."""
    n = basis.shape[1]
    xi = torch.arange(n, dtype=torch.float64, device=coeffs.device) * (2 * np.pi / n)
    y = coeffs @ basis.to(coeffs.device)
    return torch.cat([xi, y, torch.zeros(n, dtype=torch.float64, device=coeffs.device)])
