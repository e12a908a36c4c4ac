"""ctypes binding of libsfd.so (include/sfd.h).

The binding fails loudly when the compiled library is absent: there is no CPU
fallback anywhere in the product path.
"""
from __future__ import annotations

import ctypes
import os
import re
from ctypes import POINTER, c_bool, c_char_p, c_double, c_int, c_longlong, c_size_t, c_uint, c_void_p

from . import build as _build

WATER = 0
HELIUM = 1
PRECISION_FP64 = 0
PRECISION_MIXED = 1

STATUS_NONFINITE = 0x1
STATUS_PIVOT_SWAP = 0x2
STATUS_ZERO_PIVOT = 0x4
STATUS_REFINE_STALL = 0x8
STATUS_TIMEOUT = 0x20
PROFILE_CLASSES = 23


class SfdProblem(ctypes.Structure):
    _fields_ = [("physics", c_int), ("infinite_depth", c_int), ("rho", c_double), ("depth", c_double),
                ("A3", c_double), ("gravity", c_double), ("U", c_double), ("kappa", c_double),
                ("use_expansions", c_int), ("expansion_order", c_int)]


class SfdOptions(ctypes.Structure):
    _fields_ = [("precision", c_int), ("refine_iters", c_int), ("refactor_every", c_int),
                ("use_graphs", c_int), ("device", c_int), ("tensor_cores", c_int), ("pre_iters", c_int),
                ("precond_half", c_int), ("autotune", c_int), ("refactor_lag", c_int), ("extra_iters", c_int),
                ("refine_tol", c_double)]


class SimProperties(ctypes.Structure):
    """ExportTypes.cuh:8-20 (the field order the reference's rhs.py binds)."""
    _fields_ = [("L", c_double), ("rho", c_double), ("kappa", c_double), ("depth", c_double),
                ("use_expansions", c_bool), ("expansion_order", c_int), ("infinite_depth", c_bool)]


class RK4SolverOptions(ctypes.Structure):
    """ExportTypes.cuh:35-40."""
    _fields_ = [("timeStep", c_double), ("t0", c_double), ("t1", c_double), ("returnTrajectory", c_bool)]


class SfdDrive(ctypes.Structure):
    """sfd_drive (include/sfd.h): nondimensional optomechanical drive."""
    _fields_ = [(k, c_double) for k in ("detuning", "gamma", "G", "tau", "max_intensity", "x0", "sigma", "beta",
                                        "damping", "strength")] + [("augmented", c_int)]


class COptomechanicalVariables(ctypes.Structure):
    """ExportTypes.cuh:41-63 (SI units; the field order rhs.py binds)."""
    _fields_ = [(k, c_double) for k in ("detuning", "gamma", "G", "tau", "max_intensity", "initial_time",
                                        "location_x0_mode", "sigma_optical_mode", "beta", "damping_strength")]


class SfdRkf45Options(ctypes.Structure):
    _fields_ = [("atol", c_double), ("rtol", c_double), ("h_min", c_double), ("h_max", c_double),
                ("h0", c_double), ("max_rejected", c_longlong)]


class SfdRkf45Result(ctypes.Structure):
    _fields_ = [("status", c_int), ("accepted", c_longlong), ("rejected", c_longlong), ("t", c_double),
                ("h", c_double)]


class GaussLegendreOptions(ctypes.Structure):
    """ExportTypes.cuh:21-34 (the field order rhs.py's CGaussLegendreProperties binds)."""
    _fields_ = [("t0", c_double), ("t1", c_double), ("stepSize", c_double), ("newtonTolerance", c_double),
                ("maxNewtonIterations", c_size_t), ("allowSimplifiedFallback", c_bool),
                ("returnTrajectory", c_bool), ("armijo_c", c_double), ("backtrack", c_double),
                ("minAlpha", c_double), ("maxStepsHalves", c_size_t)]


class SfdGl2Options(ctypes.Structure):
    _fields_ = [("step", c_double), ("newton_tol", c_double), ("max_newton", c_longlong),
                ("allow_simplified", c_int), ("armijo_c", c_double), ("backtrack", c_double),
                ("min_alpha", c_double), ("max_halvings", c_longlong), ("fd_eps", c_double), ("jacobian", c_int)]


class SfdGl2Result(ctypes.Structure):
    _fields_ = [("status", c_int), ("steps", c_longlong), ("newton_iters", c_longlong), ("rhs_evals", c_longlong),
                ("jacobians", c_longlong), ("halvings", c_longlong), ("t", c_double), ("h", c_double),
                ("residual", c_double)]


GL2_JACOBIAN_AUTO, GL2_JACOBIAN_FD, GL2_JACOBIAN_EXACT = 0, 1, 2

_dp = POINTER(c_double)
_SIGS = {
    "sfd_default_options": (None, [POINTER(SfdOptions)]),
    "sfd_default_problem": (None, [POINTER(SfdProblem)]),
    "sfd_create": (c_int, [POINTER(c_int), c_int, POINTER(SfdProblem), c_int, POINTER(SfdOptions), POINTER(c_void_p)]),
    "sfd_destroy": (c_int, [c_void_p]),
    "sfd_set_stream": (c_int, [c_void_p, c_void_p]),
    "sfd_total_nodes": (c_int, [c_void_p]),
    "sfd_set_state_host": (c_int, [c_void_p, _dp, _dp, _dp]),
    "sfd_get_state_host": (c_int, [c_void_p, _dp, _dp, _dp]),
    "sfd_set_state_device": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "sfd_get_state_device": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "sfd_state_device_ptr": (c_int, [c_void_p, POINTER(c_void_p)]),
    "sfd_rhs_host": (c_int, [c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]),
    "sfd_rhs_device": (c_int, [c_void_p, c_void_p, c_void_p]),
    "sfd_rk4_steps": (c_int, [c_void_p, c_double, c_int]),
    "sfd_rk4_steps_async": (c_int, [c_void_p, c_double, c_int]),
    "sfd_synchronize": (c_int, [c_void_p]),
    "sfd_invariants": (c_int, [c_void_p, c_double, _dp]),
    "sfd_get_status": (c_int, [c_void_p, POINTER(c_uint), _dp, _dp]),
    "sfd_clear_status": (c_int, [c_void_p]),
    "sfd_get_refinement": (c_int, [c_void_p, _dp, POINTER(c_longlong), POINTER(c_longlong)]),
    "sfd_dense_solver_create": (c_int, [c_int, c_int, POINTER(c_void_p)]),
    "sfd_dense_solver_set_stream": (c_int, [c_void_p, c_void_p]),
    "sfd_dense_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, POINTER(c_uint)]),
    "sfd_dense_solver_destroy": (c_int, [c_void_p]),
    "sfd_kernel_launches": (c_longlong, [c_void_p]),
    "sfd_profile": (c_int, [c_void_p, c_int]),
    "sfd_profile_read": (c_int, [c_void_p, _dp, POINTER(c_longlong), c_int]),
    "sfd_profile_class_name": (c_char_p, [c_int]),
    "sfd_last_error": (c_char_p, []),
    "sfd_version": (c_char_p, []),
    "sfd_set_default_precision": (c_int, [c_int]),
    "sfd_rhs_device_noalloc": (c_int, [POINTER(SfdProblem), c_int, c_void_p, c_void_p, c_void_p]),
    "sfd_set_problem": (c_int, [c_void_p, c_int, POINTER(SfdProblem)]),
    "sfd_get_tuning": (c_int, [c_void_p, POINTER(c_int)]),
    "sfd_create_driven": (c_int, [POINTER(c_int), c_int, POINTER(SfdProblem), POINTER(SfdDrive), c_int,
                                  POINTER(SfdOptions), POINTER(c_void_p)]),
    "sfd_set_aux_host": (c_int, [c_void_p, _dp]),
    "sfd_get_aux_host": (c_int, [c_void_p, _dp]),
    "calculateRhsAugmentedOptomechanical": (c_int, [_dp, _dp, POINTER(SimProperties),
                                                    POINTER(COptomechanicalVariables), c_size_t]),
    "integrateAugmentedOptomechanicalSimulationRK4": (c_int, [_dp, POINTER(_dp), POINTER(c_size_t), POINTER(_dp),
                                                              POINTER(c_size_t), POINTER(SimProperties),
                                                              POINTER(RK4SolverOptions),
                                                              POINTER(COptomechanicalVariables), c_size_t]),
    "integrateAugmentedOptomechanicalSimulationRK4_freeMemory": (c_int, [_dp, _dp]),
    "sfd_rhs_vjp_device": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, _dp]),
    "sfd_rk4_record": (c_int, [c_void_p, c_double, c_int, c_int, _dp, _dp]),
    "sfd_rk4_vjp": (c_int, [c_void_p, _dp, _dp, _dp]),
    "sfd_adjoint_residual": (c_int, [c_void_p, _dp, POINTER(c_int)]),
    "sfd_jacobian_device": (c_int, [c_void_p, c_void_p, c_void_p]),
    "sfd_default_rkf45_options": (None, [POINTER(SfdRkf45Options)]),
    "sfd_rkf45_evolve": (c_int, [c_void_p, c_double, c_double, POINTER(SfdRkf45Options), POINTER(SfdRkf45Result),
                                 _dp, c_longlong]),
    "calculateJacobian": (c_int, [_dp, _dp] + [c_double] * 5 + [c_size_t]),
    "calculateRHSFromVectors": (c_int, [_dp] * 6 + [c_double] * 4 + [c_size_t]),
    "calculateRHS256FromVectors": (c_int, [_dp] * 6 + [c_double] * 4),
    "calculateRHS2048FromVectors": (c_int, [_dp] * 6 + [c_double] * 4),
    "calculateRHS256FromVectorsBatched": (c_int, [_dp] * 6 + [c_double] * 4 + [c_int]),
    "calculateVorticities256FromVectors": (c_int, [_dp] * 5 + [c_double] * 4),
    "calculateDerivativeFFT256": (c_int, [_dp, _dp]),
    "calculatePerturbedStates256": (c_int, [_dp] * 4 + [c_double] * 5),
    "calculateRHS256FromFile": (c_int, [ctypes.c_char_p, ctypes.c_char_p] + [c_double] * 4),
    "integrateSimulationRK4": (c_int, [_dp, POINTER(_dp), POINTER(c_size_t), POINTER(_dp), POINTER(c_size_t),
                                       POINTER(SimProperties), POINTER(RK4SolverOptions), c_size_t]),
    "integrateSimulationRK4_freeMemory": (c_int, [_dp, _dp]),
    "sfd_default_gl2_options": (None, [POINTER(SfdGl2Options)]),
    "sfd_join_background": (c_int, [c_void_p]),
    "sfd_rk4_steps_host": (c_int, [c_void_p, _dp, _dp, _dp, c_double, c_int]),
    "sfd_gl2_evolve": (c_int, [c_void_p, c_double, c_double, POINTER(SfdGl2Options), POINTER(SfdGl2Result), _dp, _dp,
                               c_longlong]),
    "sfd_gl2_evolve_cb": (c_int, [c_void_p, c_double, c_double, POINTER(SfdGl2Options), POINTER(SfdGl2Result),
                                  c_void_p, c_void_p]),
    "integrateSimulationGL2": (c_int, [_dp, POINTER(_dp), POINTER(c_size_t), POINTER(_dp), POINTER(c_size_t),
                                       POINTER(SimProperties), POINTER(GaussLegendreOptions), c_size_t]),
    "integrateSimulationGL2_freeMemory": (c_int, [_dp, _dp]),
}

_lib = None


def header_symbols() -> list[str]:
    """Function names declared in include/sfd.h."""
    txt = open(os.path.join(_build.ROOT, "include", "sfd.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"^\s*typedef\b.*?;", "", txt, flags=re.S | re.M)  # function-pointer and struct typedefs
    names = re.findall(r"^\s*(?:[A-Za-z_][A-Za-z0-9_]*[\s*]+)+([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "return")))


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) libsfd.so and bind every export."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path) or not _build.up_to_date():
        if not build_if_missing:
            raise RuntimeError(f"libsfd.so not built at {path}; run superfluid_dynamics_gb300.build.build()")
        _build.build()
    _lib = bind(ctypes.CDLL(path))
    return _lib


def bind(L: ctypes.CDLL) -> ctypes.CDLL:
    """Set the argument and result types of every export on a loaded copy of
    the library (ctypes cannot pass Python floats to an unbound function)."""
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


class SfdError(RuntimeError):
    pass


def check(rc: int) -> None:
    if rc != 0:
        msg = load().sfd_last_error()
        raise SfdError(f"sfd error {rc}: {msg.decode() if msg else ''}")
