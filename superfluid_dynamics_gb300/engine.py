"""Host-side interface over the C ABI.

`Engine` owns one batch of surfaces resident on the GPU.  The classes below it
mirror the reference's C++ solver/stepper interface so code written against the
reference reads the same here:

  reference (CuSuperHelium/CuSuperHelium)              here
  -------------------------------------------------    ---------------------------------
  WaterBoundaryProblem<N,B>   (WaterBoundaryProblem.cuh:7-40)    WaterBoundaryProblem
  HeliumBoundaryProblem<N,B>  (HeliumBoundaryProblem.cuh:6-47)   HeliumBoundaryProblem
  BaseBoundaryIntegralCalculator<N,B>::run / calculateVorticities
                              (BaseBoundaryIntegrator.cuh:137-314) BoundaryIntegralCalculator
  AutonomousRungeKuttaStepper<std_complex,2N>
                              (AutonomousRungeKuttaStepper.cuh:24-437) AutonomousRungeKuttaStepper
  SimulationManager (Python/integration/rhs.py:68-365)            SimulationManager

Arrays are float64 numpy arrays (host) or device pointers (ints) for the
device-side calls.  Errors raise SfdError; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import HELIUM, PRECISION_FP64, PRECISION_MIXED, WATER, SfdError, check


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


@dataclass
class Physics:
    """Nondimensional physics of one surface (sfd_problem)."""

    physics: int = WATER
    rho: float = 0.0
    depth: float = 1.0
    A3: float | None = None        # None: the reference's h^4 / 3
    gravity: float = 1.0
    U: float = 0.0
    kappa: float = 0.0
    infinite_depth: bool = False
    use_expansions: bool = False
    expansion_order: int = 1

    def to_c(self) -> _lib.SfdProblem:
        return _lib.SfdProblem(self.physics, 1 if self.infinite_depth else 0, self.rho, self.depth,
                               self.A3 if self.A3 is not None else 0.0, self.gravity, self.U, self.kappa,
                               1 if self.use_expansions else 0, self.expansion_order)


@dataclass
class Drive:
    """Optomechanical drive of a helium film, nondimensional (sfd_drive).

    I(y, x) = gamma^2 max_intensity / 4 / ((detuning - G y)^2 + (gamma/2)^2) exp(-(x - x0)^2 / (2 sigma^2));
    dphi/dt += damping * v + strength * I, and with `augmented` the state gains
    the delayed intensity D: dphi/dt += D, dD/dt = beta I - D / tau
    (HeliumDrivenAutonomousProblem.cuh, DelayedIntensityIntegrator.cuh)."""

    detuning: float = 0.0
    gamma: float = 1.0
    G: float = 1.0
    tau: float = 1.0
    max_intensity: float = 0.0
    x0: float = 0.0
    sigma: float = 1.0
    beta: float = 0.0
    damping: float = 0.0
    strength: float = 0.0
    augmented: bool = True

    def to_c(self) -> _lib.SfdDrive:
        return _lib.SfdDrive(self.detuning, self.gamma, self.G, self.tau, self.max_intensity, self.x0, self.sigma,
                             self.beta, self.damping, self.strength, 1 if self.augmented else 0)


@dataclass
class Options:
    """Engine options (sfd_options of include/sfd.h).

    precision      PRECISION_MIXED (FP32 / tensor-core preconditioner with
                   double-float refinement) or PRECISION_FP64 (blocked FP64 LU)
    refine_iters   mixed: FP32 corrections after the double-float residual
    refactor_every mixed: rebuild the preconditioner every k RK4 steps
    use_graphs     capture one RK4 step in a CUDA graph
    tensor_cores   mixed: Gauss-Jordan update on tcgen05 (else SIMT)
    pre_iters      mixed: FP32 full-residual iterations before the accurate pass
    precond_half   mixed: apply the preconditioner from its FP16 copy
    autotune       time the boundary-sum CTA shapes on the first steps
    refactor_lag   mixed, stepping: rebuild on a side stream and switch k steps
                   later (0 < k < refactor_every; 0 rebuilds inside the step)
    extra_iters    extra corrections of the solve (0..4), run only where the
                   relative residual is above refine_tol
    refine_tol     relative residual tolerance max|phi' - M a| / max|phi'|
                   (<= 0: no check)
    """
    precision: int = PRECISION_MIXED
    refine_iters: int = 2
    refactor_every: int = 1
    use_graphs: bool = True
    device: int = 0
    tensor_cores: bool = True
    pre_iters: int = 1
    precond_half: bool = True
    autotune: bool = True
    refactor_lag: int = 0
    extra_iters: int = 2
    refine_tol: float = 1e-10

    def to_c(self) -> _lib.SfdOptions:
        return _lib.SfdOptions(self.precision, self.refine_iters, self.refactor_every,
                               1 if self.use_graphs else 0, self.device, 1 if self.tensor_cores else 0,
                               self.pre_iters, 1 if self.precond_half else 0, 1 if self.autotune else 0,
                               self.refactor_lag, self.extra_iters, float(self.refine_tol))


class Engine:
    """A batch of surfaces (possibly of different N) resident in device memory."""

    def __init__(self, n, physics: Physics | list[Physics] | None = None, options: Options | None = None,
                 drive: Drive | list[Drive] | None = None):
        L = _lib.load()
        ns = [int(n)] if np.isscalar(n) else [int(v) for v in n]
        if physics is None:
            physics = Physics()
        shared = not isinstance(physics, (list, tuple))
        probs = [physics] if shared else list(physics)
        if not shared and len(probs) != len(ns):
            raise ValueError("one Physics per surface required")
        carr = (_lib.SfdProblem * len(probs))(*[p.to_c() for p in probs])
        narr = (ctypes.c_int * len(ns))(*ns)
        opt = (options or Options()).to_c()
        h = ctypes.c_void_p()
        if drive is None:
            check(L.sfd_create(narr, len(ns), carr, 1 if shared else 0, ctypes.byref(opt), ctypes.byref(h)))
        else:
            drs = [drive] if shared else (list(drive) if isinstance(drive, (list, tuple)) else [drive] * len(ns))
            darr = (_lib.SfdDrive * len(drs))(*[d.to_c() for d in drs])
            check(L.sfd_create_driven(narr, len(ns), carr, darr, 1 if shared else 0, ctypes.byref(opt),
                                      ctypes.byref(h)))
        self.augmented = drive is not None and any(
            d.augmented for d in ([drive] if isinstance(drive, Drive) else drive))
        self._h = h
        self._L = L
        self.sizes = ns
        self.ntot = int(sum(ns))
        self.nsurf = len(ns)
        self.offsets = np.concatenate([[0], np.cumsum(ns)]).astype(np.int64)
        self.options = options or Options()

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.sfd_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state
    def set_state(self, x, y, phi) -> None:
        x, y, phi = _f64(x), _f64(y), _f64(phi)
        if x.size != self.ntot or y.size != self.ntot or phi.size != self.ntot:
            raise ValueError(f"state arrays must hold {self.ntot} nodes")
        check(self._L.sfd_set_state_host(self._h, _dp(x), _dp(y), _dp(phi)))

    def get_state(self):
        x, y, phi = (np.empty(self.ntot) for _ in range(3))
        check(self._L.sfd_get_state_host(self._h, _dp(x), _dp(y), _dp(phi)))
        return x, y, phi

    def set_aux(self, D) -> None:
        """Delayed-intensity block of an augmented driven engine."""
        D = _f64(D)
        if D.size != self.ntot:
            raise ValueError(f"the delayed intensity must hold {self.ntot} nodes")
        check(self._L.sfd_set_aux_host(self._h, _dp(D)))

    def get_aux(self) -> np.ndarray:
        D = np.empty(self.ntot)
        check(self._L.sfd_get_aux_host(self._h, _dp(D)))
        return D

    def set_state_device(self, x_ptr: int, y_ptr: int, phi_ptr: int) -> None:
        check(self._L.sfd_set_state_device(self._h, x_ptr, y_ptr, phi_ptr))

    def get_state_device(self, x_ptr: int, y_ptr: int, phi_ptr: int) -> None:
        check(self._L.sfd_get_state_device(self._h, x_ptr, y_ptr, phi_ptr))

    def state_device_ptr(self) -> int:
        p = ctypes.c_void_p()
        check(self._L.sfd_state_device_ptr(self._h, ctypes.byref(p)))
        return int(p.value)

    # -- evaluation
    def rhs(self, diagnostics: bool = False):
        """RHS of the resident state: (dx, dy, dphi)[, a, zp, zpp]."""
        dx, dy, dphi, a = (np.empty(self.ntot) for _ in range(4))
        zp = np.empty(self.ntot, np.complex128)
        zpp = np.empty(self.ntot, np.complex128)
        check(self._L.sfd_rhs_host(self._h, _dp(dx), _dp(dy), _dp(dphi), _dp(a),
                                   zp.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   zpp.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        if diagnostics:
            return dx, dy, dphi, a, zp, zpp
        return dx, dy, dphi

    def rhs_device(self, state_ptr: int, out_ptr: int) -> None:
        check(self._L.sfd_rhs_device(self._h, state_ptr, out_ptr))

    def step(self, dt: float, steps: int = 1, sync: bool = True) -> None:
        fn = self._L.sfd_rk4_steps if sync else self._L.sfd_rk4_steps_async
        check(fn(self._h, float(dt), int(steps)))

    def step_host(self, x: np.ndarray, y: np.ndarray, phi: np.ndarray, dt: float, steps: int = 1) -> None:
        """Copy the host state in, run `steps` RK4 steps and copy it back into
        the same float64 arrays (one call, one synchronisation)."""
        for a in (x, y, phi):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != self.ntot:
                raise ValueError(f"state arrays must be contiguous float64 of {self.ntot} nodes")
        check(self._L.sfd_rk4_steps_host(self._h, _dp(x), _dp(y), _dp(phi), float(dt), int(steps)))

    def evolve_rkf45(self, t0: float, t1: float, atol: float = 1e-6, rtol: float = 1e-3, h_min: float = 1e-16,
                     h_max: float = 1e10, h0: float = 1e-2, max_rejected: int = 500, max_times: int = 1 << 20):
        """Adaptive Runge-Kutta-Fehlberg 4(5) of the resident state from t0 to t1
        (the reference's RK45Base).  Returns (result dict, times of the accepted steps)."""
        o = _lib.SfdRkf45Options(atol, rtol, h_min, h_max, h0, max_rejected)
        r = _lib.SfdRkf45Result()
        times = np.zeros(max_times)
        check(self._L.sfd_rkf45_evolve(self._h, float(t0), float(t1), ctypes.byref(o), ctypes.byref(r),
                                       _dp(times), max_times))
        res = {"status": r.status, "accepted": r.accepted, "rejected": r.rejected, "t": r.t, "h": r.h}
        return res, times[:min(r.accepted, max_times)].copy()

    def evolve_gl2(self, t0: float, t1: float, step: float = 0.01, newton_tol: float = 1e-10, max_newton: int = 20,
                   allow_simplified: bool = False, armijo_c: float = 1e-4, backtrack: float = 0.5,
                   min_alpha: float = 1e-6, max_halvings: int = 6, fd_eps: float = 1e-6,
                   jacobian: str = "auto", max_steps: int = 1 << 16, record_states: bool = False):
        """Implicit two-stage Gauss-Legendre of the resident state from t0 to t1
        (the reference's GaussLegendre2).  jacobian: "auto", "fd" or "exact".
        Returns (result dict, times of the accepted steps[, states after them])."""
        mode = {"auto": _lib.GL2_JACOBIAN_AUTO, "fd": _lib.GL2_JACOBIAN_FD, "exact": _lib.GL2_JACOBIAN_EXACT}[jacobian]
        o = _lib.SfdGl2Options(step, newton_tol, max_newton, 1 if allow_simplified else 0, armijo_c, backtrack,
                               min_alpha, max_halvings, fd_eps, mode)
        r = _lib.SfdGl2Result()
        times = np.zeros(max_steps)
        states = np.zeros((max_steps, 3 * self.ntot)) if record_states else None
        check(self._L.sfd_gl2_evolve(self._h, float(t0), float(t1), ctypes.byref(o), ctypes.byref(r), _dp(times),
                                     _dp(states) if record_states else None, max_steps))
        res = {k: getattr(r, k) for k, _ in _lib.SfdGl2Result._fields_}
        k = min(r.steps, max_steps)
        if record_states:
            return res, times[:k].copy(), states[:k].copy()
        return res, times[:k].copy()

    def synchronize(self) -> None:
        check(self._L.sfd_synchronize(self._h))

    def join_background(self) -> None:
        """Make the engine stream wait for an in-flight background rebuild."""
        check(self._L.sfd_join_background(self._h))

    def invariants(self, kappa: float = 0.0) -> np.ndarray:
        out = np.empty(5 * self.nsurf)
        check(self._L.sfd_invariants(self._h, float(kappa), _dp(out)))
        return out.reshape(self.nsurf, 5)

    def status(self):
        st = (ctypes.c_uint * self.nsurf)()
        lm = np.empty(self.nsurf)
        rn = np.empty(self.nsurf)
        check(self._L.sfd_get_status(self._h, st, _dp(lm), _dp(rn)))
        return np.array(list(st), dtype=np.uint32), lm, rn

    def clear_status(self) -> None:
        check(self._L.sfd_clear_status(self._h))

    def refinement(self) -> dict:
        """Refinement record since the last clear_status: per-surface max final
        relative residual and extra corrections run, and the preconditioner
        rebuilds a refinement stall triggered."""
        rel = np.empty(self.nsurf)
        extra = (ctypes.c_longlong * self.nsurf)()
        rb = ctypes.c_longlong(0)
        check(self._L.sfd_get_refinement(self._h, _dp(rel), extra, ctypes.byref(rb)))
        return {"rel_residual": rel, "extra_iters": np.array(list(extra), dtype=np.int64),
                "stall_rebuilds": int(rb.value)}

    def set_stream(self, stream_ptr: int) -> None:
        check(self._L.sfd_set_stream(self._h, stream_ptr))

    def profile(self, enable: bool = True) -> None:
        """Per-kernel-class CUDA-event timing (steps run without graphs meanwhile)."""
        check(self._L.sfd_profile(self._h, 1 if enable else 0))

    def profile_read(self) -> dict:
        n = _lib.PROFILE_CLASSES
        ms = np.zeros(n)
        cnt = (ctypes.c_longlong * n)()
        check(self._L.sfd_profile_read(self._h, _dp(ms), cnt, n))
        return {self._L.sfd_profile_class_name(i).decode(): (float(ms[i]), int(cnt[i])) for i in range(n)}

    @property
    def kernel_launches(self) -> int:
        return int(self._L.sfd_kernel_launches(self._h))

    def tuning(self) -> dict:
        """Boundary-sum source groups per CTA in use, by pass precision."""
        g = (ctypes.c_int * 3)()
        check(self._L.sfd_get_tuning(self._h, g))
        return {"fp64": g[0], "df": g[1], "fp32": g[2]}

    def set_problem(self, physics: Physics, surface: int = 0) -> None:
        """Replace one surface's parameters (A3, g, ...) in place."""
        check(self._L.sfd_set_problem(self._h, int(surface), ctypes.byref(physics.to_c())))

    # -------------------------------------------------------------- reverse mode
    # Engines with one surface (water rho = 0 or helium, standard closure):
    # FP64 (LU records) or mixed with the FP16 preconditioner (refinement
    # preconditioned by its transpose).
    def rhs_vjp_device(self, state_ptr: int, cot_ptr: int, grad_ptr: int) -> float:
        """grad = J(state)^T cot on device arrays of 3n doubles; returns the
        parameter derivative (d/dA3 helium, d/dg water)."""
        gp = np.zeros(1)
        check(self._L.sfd_rhs_vjp_device(self._h, state_ptr, cot_ptr, grad_ptr, _dp(gp)))
        return float(gp[0])

    def rhs_vjp(self, state: np.ndarray, cot: np.ndarray):
        """Host convenience over rhs_vjp_device (device buffers from torch)."""
        import torch
        state, cot = _f64(state), _f64(cot)
        self._check_state_size(state, cot)
        dev = torch.device("cuda", self.options.device)
        s = torch.as_tensor(state, device=dev)
        c = torch.as_tensor(cot, device=dev)
        g = torch.empty_like(s)
        gp = self.rhs_vjp_device(s.data_ptr(), c.data_ptr(), g.data_ptr())
        return g.cpu().numpy(), gp

    def jacobian(self, state: np.ndarray) -> np.ndarray:
        """Exact RHS Jacobian J[row, col] at state = [x|y|phi] (reverse sweeps, FP64 engine, one surface)."""
        import torch
        state = _f64(state)
        self._check_state_size(state)
        dev = torch.device("cuda", self.options.device)
        s = torch.as_tensor(state, device=dev)
        j = torch.empty(s.numel() * s.numel(), dtype=torch.float64, device=dev)
        check(self._L.sfd_jacobian_device(self._h, s.data_ptr(), j.data_ptr()))
        n3 = s.numel()
        return j.cpu().numpy().reshape(n3, n3).T.copy()

    def rk4_record(self, dt: float, steps: int, checkpoint_every: int, state0: np.ndarray) -> np.ndarray:
        """Integrate from state0 = [x|y|phi] keeping checkpoints; returns the final state."""
        s0 = _f64(state0)
        self._check_state_size(s0)
        out = np.empty_like(s0)
        check(self._L.sfd_rk4_record(self._h, float(dt), int(steps), int(checkpoint_every), _dp(s0), _dp(out)))
        return out

    def rk4_vjp(self, cot_final: np.ndarray):
        """(d final / d state0)^T cot_final and the parameter derivative of <cot_final, final>."""
        c = _f64(cot_final)
        self._check_state_size(c)
        g = np.empty_like(c)
        gp = np.zeros(1)
        check(self._L.sfd_rk4_vjp(self._h, _dp(c), _dp(g), _dp(gp)))
        return g, float(gp[0])

    def adjoint_residual(self) -> tuple[float, int]:
        """Mixed engines: the largest final relative residual of the transposed
        solves of the last reverse-mode call, and the most preconditioner
        products one of them ran ((0.0, 0) for FP64 engines)."""
        rel = np.zeros(1)
        corr = ctypes.c_int(0)
        check(self._L.sfd_adjoint_residual(self._h, _dp(rel), ctypes.byref(corr)))
        return float(rel[0]), int(corr.value)

    def _check_state_size(self, *arrays) -> None:
        """Reverse-mode arrays hold the full state [x | y | phi]: the library
        reads (and the Jacobian writes) exactly that many values."""
        n3 = 3 * self.ntot
        for a in arrays:
            if a.size != n3:
                raise ValueError(f"state-sized arrays must hold 3 * {self.ntot} = {n3} values, not {a.size}")

    def split(self, arr: np.ndarray) -> list[np.ndarray]:
        return [arr[self.offsets[i]:self.offsets[i + 1]] for i in range(self.nsurf)]


# ------------------------------------------------------------------ reference-shaped classes
class WaterBoundaryProblem(Physics):
    """Gravity water waves (WaterBoundaryProblem.cuh:7-40); rho is the density ratio."""

    def __init__(self, rho: float = 0.0, gravity: float = 1.0):
        super().__init__(physics=WATER, rho=rho, gravity=gravity)


class HeliumBoundaryProblem(Physics):
    """Finite-depth helium film (HeliumBoundaryProblem.cuh:6-47); A3 None = h^4/3."""

    def __init__(self, depth: float, A3: float | None = None, infinite_depth: bool = False, kappa: float = 0.0,
                 use_expansions: bool = False, expansion_order: int = 1):
        super().__init__(physics=HELIUM, depth=depth, A3=A3, infinite_depth=infinite_depth, kappa=kappa,
                         use_expansions=use_expansions, expansion_order=expansion_order)


class BoundaryIntegralCalculator:
    """run(state) -> rhs, with state / rhs laid out as the reference's real
    adapter does (RealBoundaryIntegralCalculator.cuh:4-23): [x | y | phi]."""

    def __init__(self, N: int, problem: Physics, options: Options | None = None, batch: int = 1):
        self.N = N
        self.batch = batch
        self.engine = Engine([N] * batch, problem, options)

    def run(self, state: np.ndarray) -> np.ndarray:
        n = self.N * self.batch
        state = _f64(state)
        self.engine.set_state(state[:n], state[n:2 * n], state[2 * n:3 * n])
        dx, dy, dphi = self.engine.rhs()
        return np.concatenate([dx, dy, dphi])

    def calculateVorticities(self, state: np.ndarray) -> np.ndarray:
        n = self.N * self.batch
        state = _f64(state)
        self.engine.set_state(state[:n], state[n:2 * n], state[2 * n:3 * n])
        return self.engine.rhs(diagnostics=True)[3]


class AutonomousRungeKuttaStepper:
    """Classic RK4 over a BoundaryIntegralCalculator (AutonomousRungeKuttaStepper.cuh:24-437)."""

    def __init__(self, calculator: BoundaryIntegralCalculator, tstep: float = 1e-2):
        self.calc = calculator
        self.timeStep = tstep
        self.currentTime = 0.0

    def setTimeStep(self, tstep: float) -> None:
        self.timeStep = tstep

    def initialize(self, state: np.ndarray) -> None:
        n = self.calc.N * self.calc.batch
        state = _f64(state)
        self.calc.engine.set_state(state[:n], state[n:2 * n], state[2 * n:3 * n])

    def runStep(self) -> None:
        self.calc.engine.step(self.timeStep, 1)
        self.currentTime += self.timeStep

    def runEvolution(self, startTime: float, endTime: float, log=None) -> None:
        self.currentTime = startTime
        steps = int((endTime - startTime) / self.timeStep)
        for _ in range(steps):
            self.calc.engine.step(self.timeStep, 1)
            self.currentTime += self.timeStep
            if log is not None:
                log(self.currentTime, self.state())

    def state(self) -> np.ndarray:
        return np.concatenate(self.calc.engine.get_state())


class SimulationManager:
    """The reference's ctypes front end (Python/integration/rhs.py:68-365) over
    the same exported symbols, for Linux / this library."""

    def __init__(self, dll_path: str | None = None):
        self.lib = _lib.load() if dll_path is None else _lib.bind(ctypes.CDLL(dll_path))

    def _rhs(self, fn, x, y, phi, *args, nodes=None):
        x, y, phi = _f64(x), _f64(y), _f64(phi)
        if y.shape[0] != x.shape[0] or phi.shape[0] != x.shape[0]:
            raise ValueError("Input arrays must have the same length")
        if nodes is not None and x.shape[0] != nodes:
            # the fixed-size exports read exactly this many nodes
            raise ValueError(f"Input arrays must hold {nodes} nodes")
        vx, vy, dphi = np.empty_like(x), np.empty_like(x), np.empty_like(x)
        rc = fn(_dp(x), _dp(y), _dp(phi), _dp(vx), _dp(vy), _dp(dphi), *args)
        return rc, vx, vy, dphi

    def calculate_rhs_from_vectors(self, x, y, phi, L, rho, kappa, depth):
        return self._rhs(self.lib.calculateRHSFromVectors, x, y, phi, L, rho, kappa, depth, len(x))

    def calculate_rhs256_from_vectors(self, x, y, phi, L, rho, kappa, depth):
        return self._rhs(self.lib.calculateRHS256FromVectors, x, y, phi, L, rho, kappa, depth, nodes=256)

    def calculate_rhs2048_from_vectors(self, x, y, phi, L, rho, kappa, depth):
        return self._rhs(self.lib.calculateRHS2048FromVectors, x, y, phi, L, rho, kappa, depth, nodes=2048)

    def calculate_rhs256_from_vectors_batched(self, x, y, phi, L, rho, kappa, depth, batch_size):
        # rhs.py:187-189 checks y and phi against 256 * batch_size
        n = len(x) // batch_size if batch_size > 0 else 0
        if batch_size <= 0 or len(y) != n * batch_size or len(phi) != 256 * batch_size or len(x) != 256 * batch_size:
            raise ValueError("Input arrays must have the same length equal to 256 * batch_size")
        return self._rhs(self.lib.calculateRHS256FromVectorsBatched, x, y, phi, L, rho, kappa, depth, batch_size)

    def calculate_vorticities256_from_vectors(self, Z, phi, L, rho, kappa, depth):
        Z = np.ascontiguousarray(Z, dtype=np.complex128)
        phi = np.ascontiguousarray(phi, dtype=np.complex128)
        if phi.shape[0] != Z.shape[0]:
            raise ValueError("Input arrays must have the same length")
        if Z.shape[0] != 256:
            raise ValueError("Input arrays must hold 256 nodes")
        a = np.empty(Z.shape[0])
        Zp = np.empty(Z.shape[0], np.complex128)
        Zpp = np.empty(Z.shape[0], np.complex128)
        cp = lambda v: v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        rc = self.lib.calculateVorticities256FromVectors(cp(Z), cp(phi), _dp(a), cp(Zp), cp(Zpp), L, rho, kappa, depth)
        return rc, a, Zp, Zpp

    def calculate_derivativeFFT256(self, inp):
        inp = np.ascontiguousarray(inp, dtype=np.complex128)
        if inp.shape[0] != 256:
            raise ValueError("Input array must hold 256 nodes")
        out = np.empty(inp.shape[0], np.complex128)
        cp = lambda v: v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        return self.lib.calculateDerivativeFFT256(cp(inp), cp(out)), out

    def integrate_simulation_rk4(self, x, y, phi, L, rho, kappa, depth, t0, t1, dt, return_trajectory=True):
        N = len(x)
        state = np.concatenate([_f64(x), _f64(y), _f64(phi)])
        sp = _lib.SimProperties(L, rho, kappa, depth, False, 1, False)
        ro = _lib.RK4SolverOptions(dt, t0, t1, return_trajectory)
        states = ctypes.POINTER(ctypes.c_double)()
        times = ctypes.POINTER(ctypes.c_double)()
        ns, nt = ctypes.c_size_t(), ctypes.c_size_t()
        rc = self.lib.integrateSimulationRK4(_dp(state), ctypes.byref(states), ctypes.byref(ns), ctypes.byref(times),
                                             ctypes.byref(nt), ctypes.byref(sp), ctypes.byref(ro), N)
        if rc != 0:
            raise SfdError(self.lib.sfd_last_error().decode())
        try:
            S = np.ctypeslib.as_array(states, shape=(ns.value, 3 * N)).copy()
            T = np.ctypeslib.as_array(times, shape=(nt.value,)).copy() if nt.value else np.empty(0)
        finally:
            self.lib.integrateSimulationRK4_freeMemory(states, times)
        return S, T

    def integrate(self, y0, sim_props: _lib.SimProperties, gl_props: _lib.GaussLegendreOptions):
        """rhs.py:224-264: GL2 integration (integrateSimulationGL2); returns
        (rc, times, states) with states[i] = [x | y | phi] after step i (the
        initial state first), or (rc, None, None) on failure."""
        y0 = _f64(y0)
        n = y0.size // 3
        states = ctypes.POINTER(ctypes.c_double)()
        times = ctypes.POINTER(ctypes.c_double)()
        ns, nt = ctypes.c_size_t(), ctypes.c_size_t()
        rc = self.lib.integrateSimulationGL2(_dp(y0), ctypes.byref(states), ctypes.byref(ns), ctypes.byref(times),
                                             ctypes.byref(nt), ctypes.byref(sim_props), ctypes.byref(gl_props), n)
        if rc != 0:
            return rc, None, None
        try:
            S = np.ctypeslib.as_array(states, shape=(ns.value, 3 * n)).copy()
            T = np.ctypeslib.as_array(times, shape=(nt.value,)).copy() if nt.value else np.empty(0)
        finally:
            self.lib.integrateSimulationGL2_freeMemory(states, times)
        return rc, T, S

    def calculate_rhs256(self, input_file: str, output_file: str, L, rho, kappa, depth) -> int:
        """rhs.py:91-99: RHS of the 256-node state file `input_file`, written to
        `output_file` as a state file (calculateRHS256FromFile)."""
        return self.lib.calculateRHS256FromFile(os.fsencode(input_file), os.fsencode(output_file), L, rho, kappa,
                                                depth)

    def calculate_perturbed_states256(self, x, y, phi, L, rho, kappa, depth, epsilon=1e-6):
        """rhs.py:197-211: (rc, Zperturbed), the 6 N^2 complex values of the 3N
        perturbed states at N = 256 (calculatePerturbedStates256)."""
        x, y, phi = _f64(x), _f64(y), _f64(phi)
        if y.shape[0] != x.shape[0] or phi.shape[0] != x.shape[0]:
            raise ValueError("Input arrays must have the same length")
        if x.shape[0] != 256:
            raise ValueError("Input arrays must hold 256 nodes")
        n = x.shape[0]
        Z = np.empty(6 * n * n, dtype=np.complex128)
        rc = self.lib.calculatePerturbedStates256(_dp(x), _dp(y), _dp(phi),
                                                  Z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), L, rho, kappa,
                                                  depth, epsilon)
        return rc, Z

    def calculate_jacobian(self, x, y, phi, L, rho, kappa, depth, epsilon=1e-6):
        """rhs.py:213-222: (rc, J) with J[row, col] = d rhs_row / d state_col, a
        Fortran-ordered [3N x 3N] array as the export writes it (column-major)."""
        n = len(x)
        if len(y) != n or len(phi) != n:
            raise ValueError("Input arrays must have the same length")
        state = np.concatenate([_f64(x), _f64(y), _f64(phi)])
        J = np.empty((3 * n, 3 * n), dtype=np.float64, order="F")
        rc = self.lib.calculateJacobian(_dp(state), J.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), L, rho, kappa,
                                        depth, epsilon, n)
        return rc, J

    def calculate_augmented_rhs(self, y0, sim_props: _lib.SimProperties, opt_props: _lib.COptomechanicalVariables):
        """rhs.py:348-358: RHS of [x | y | phi | D] for the augmented driven film (SI inputs)."""
        y0 = _f64(y0)
        rhs = np.empty_like(y0)
        rc = self.lib.calculateRhsAugmentedOptomechanical(_dp(y0), _dp(rhs), ctypes.byref(sim_props),
                                                          ctypes.byref(opt_props), y0.size // 4)
        if rc != 0:
            raise SfdError(self.lib.sfd_last_error().decode())
        return rhs

    def integrate_augmented_optomechanical_problem(self, y0, sim_props: _lib.SimProperties,
                                                   opt_props: _lib.COptomechanicalVariables,
                                                   rk4_props: _lib.RK4SolverOptions):
        """rhs.py:306-346: returns (rc, times, states) with states [steps + 1, 4N]."""
        y0 = _f64(y0)
        states = ctypes.POINTER(ctypes.c_double)()
        times = ctypes.POINTER(ctypes.c_double)()
        ns, nt = ctypes.c_size_t(), ctypes.c_size_t()
        rc = self.lib.integrateAugmentedOptomechanicalSimulationRK4(
            _dp(y0), ctypes.byref(states), ctypes.byref(ns), ctypes.byref(times), ctypes.byref(nt),
            ctypes.byref(sim_props), ctypes.byref(rk4_props), ctypes.byref(opt_props), y0.size // 4)
        if rc != 0:
            return rc, None, None
        try:
            S = np.ctypeslib.as_array(states, shape=(ns.value, y0.size)).copy()
            T = np.ctypeslib.as_array(times, shape=(nt.value,)).copy() if nt.value else np.empty(0)
        finally:
            self.lib.integrateAugmentedOptomechanicalSimulationRK4_freeMemory(states, times)
        return rc, T, S
