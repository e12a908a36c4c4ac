"""ctypes front end of the CPU FP64 oracle (sfd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, always as the checker.  The product library never
imports this module.

The oracle restates the reference's FP64 boundary-integral path
(CuSuperHelium/CuSuperHelium/*.cuh); each C function cites the routine it
follows.  Problems are described by :class:`Problem` (nondimensional units).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "sfd_oracle.c")
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libsfd_oracle.so")

WATER = 0
HELIUM = 1


class _CProblem(ctypes.Structure):
    _fields_ = [
        ("physics", ctypes.c_int),
        ("rho", ctypes.c_double),
        ("depth", ctypes.c_double),
        ("vdw", ctypes.c_double),
        ("gravity", ctypes.c_double),
        ("U", ctypes.c_double),
        ("infinite_depth", ctypes.c_int),
    ]


@dataclass
class Problem:
    """Nondimensional physics of one surface.

    physics: WATER (createMKernel path) or HELIUM (finite-depth path).
    A3: van der Waals constant; None means the reference's fixed h^4/3.
    """

    physics: int = WATER
    rho: float = 0.0
    depth: float = 1.0
    A3: float | None = None
    gravity: float = 1.0
    U: float = 0.0
    infinite_depth: bool = False

    @property
    def vdw(self) -> float:
        if self.A3 is None:
            return self.depth / 3.0
        return self.A3 / self.depth ** 3

    def to_c(self) -> _CProblem:
        return _CProblem(self.physics, self.rho, self.depth, self.vdw, self.gravity, self.U,
                         1 if self.infinite_depth else 0)


class _CDrive(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("detuning", "gamma", "G", "tau", "max_intensity", "x0", "sigma",
                                                 "beta", "damping", "strength")] + [("augmented", ctypes.c_int)]


@dataclass
class Drive:
    """Optomechanical drive (nondimensional), see orc_drive in sfd_oracle.c."""

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

    def to_c(self) -> _CDrive:
        return _CDrive(self.detuning, self.gamma, self.G, self.tau, self.max_intensity, self.x0, self.sigma,
                       self.beta, self.damping, self.strength, 1 if self.augmented else 0)


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build (gcc, OpenMP, no -march flags)."""
    os.makedirs(_BUILD, exist_ok=True)
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC):
        tmp = _LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11",
                               "-o", tmp, _SRC, "-lm"])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        pp = ctypes.POINTER(_CProblem)
        L.orc_fft.argtypes = [ctypes.c_int, dp, ctypes.c_int]
        L.orc_fft_derivative.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int, ctypes.c_double]
        L.orc_zphi_derivative.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double, dp, dp, dp]
        L.orc_create_M_water.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double, dp]
        L.orc_create_M_helium.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_int, dp]
        L.orc_lu_factor.argtypes = [ctypes.c_int, dp, ip]
        L.orc_lu_factor.restype = ctypes.c_int
        L.orc_lu_solve.argtypes = [ctypes.c_int, dp, ip, dp]
        L.orc_velocities.argtypes = [ctypes.c_int, dp, dp, dp, dp, dp, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_int, dp]
        L.orc_rhs_phi_water.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_double, dp]
        L.orc_rhs_phi_helium.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double, dp]
        L.orc_rhs.argtypes = [pp, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_rhs.restype = ctypes.c_int
        L.orc_rk4_step.argtypes = [pp, ctypes.c_int, ctypes.c_double, dp, dp, dp]
        L.orc_rk4_step.restype = ctypes.c_int
        L.orc_rk4_steps.argtypes = [pp, ctypes.c_int, ctypes.c_double, ctypes.c_int, dp, dp, dp]
        L.orc_rk4_steps.restype = ctypes.c_int
        L.orc_invariants.argtypes = [pp, ctypes.c_int, dp, dp, dp, dp, dp, ctypes.c_double, dp]
        ll = ctypes.c_longlong
        L.orc_rkf45_evolve.argtypes = [pp, ctypes.c_int] + [ctypes.c_double] * 7 + [ll, dp, dp, dp, dp, dp,
                                                                                      ctypes.POINTER(ll),
                                                                                      ctypes.POINTER(ll), dp, ll]
        L.orc_rkf45_evolve.restype = ctypes.c_int
        dr = ctypes.POINTER(_CDrive)
        L.orc_intensity.argtypes = [dr, ctypes.c_double, ctypes.c_double]
        L.orc_intensity.restype = ctypes.c_double
        L.orc_rhs_driven.argtypes = [pp, dr, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_rhs_driven.restype = ctypes.c_int
        L.orc_rk4_steps_driven.argtypes = [pp, dr, ctypes.c_int, ctypes.c_double, ctypes.c_int, dp, dp, dp, dp]
        L.orc_rk4_steps_driven.restype = ctypes.c_int
        L.orc_cot_green.argtypes = [ctypes.c_double] * 4 + [dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_set_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def cot_green(zk: complex, zj: complex) -> complex:
    out = np.empty(2)
    lib().orc_cot_green(zk.real, zk.imag, zj.real, zj.imag, _dp(out))
    return complex(out[0], out[1])


def set_threads(n: int) -> int:
    return lib().orc_set_threads(int(n))


def fft(data, inverse: bool = False) -> np.ndarray:
    d = _c128(data).copy()
    lib().orc_fft(d.size, _dp(d), 1 if inverse else -1)
    return d


def fft_derivative(data, second: bool = False, scale: float = 1.0) -> np.ndarray:
    d = _c128(data)
    out = np.empty_like(d)
    lib().orc_fft_derivative(d.size, _dp(d), _dp(out), 1 if second else 0, float(scale))
    return out


def zphi_derivative(Z, Phi, rho: float = 0.0, U: float = 0.0):
    Z = _c128(Z)
    Phi = _c128(Phi)
    n = Z.size
    Zp = np.empty(n, np.complex128)
    PhP = np.empty(n, np.complex128)
    Zpp = np.empty(n, np.complex128)
    lib().orc_zphi_derivative(n, _dp(Z), _dp(Phi), rho, U, _dp(Zp), _dp(PhP), _dp(Zpp))
    return Zp, PhP, Zpp


def create_M(problem: Problem, Z, Zp, Zpp) -> np.ndarray:
    """Row-major M (row k, column j)."""
    Z, Zp, Zpp = _c128(Z), _c128(Zp), _c128(Zpp)
    n = Z.size
    M = np.empty((n, n), np.float64)
    if problem.physics == WATER:
        lib().orc_create_M_water(n, _dp(Z), _dp(Zp), _dp(Zpp), problem.rho, _dp(M))
    else:
        lib().orc_create_M_helium(n, _dp(Z), _dp(Zp), _dp(Zpp), problem.depth,
                                  1 if problem.infinite_depth else 0, _dp(M))
    return M


def lu_solve(M, b):
    A = _f64(M).copy()
    x = _f64(b).copy()
    n = x.size
    piv = np.empty(n, np.int32)
    info = lib().orc_lu_factor(n, _dp(A), piv.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    lib().orc_lu_solve(n, _dp(A), piv.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(x))
    return x, info


def velocities(problem: Problem, Z, Zp, Zpp, a, ap, lower: bool = True) -> np.ndarray:
    Z, Zp, Zpp, ap = _c128(Z), _c128(Zp), _c128(Zpp), _c128(ap)
    a = _f64(a)
    n = Z.size
    vel = np.empty(n, np.complex128)
    lib().orc_velocities(n, _dp(Z), _dp(Zp), _dp(Zpp), _dp(a), _dp(ap),
                         1 if problem.physics == HELIUM else 0, problem.depth,
                         1 if problem.infinite_depth else 0, 1 if lower else 0, _dp(vel))
    return vel


def rhs_phi_water(Z, vlow, vup, rho: float = 0.0, g: float = 1.0) -> np.ndarray:
    Z, vlow, vup = _c128(Z), _c128(vlow), _c128(vup)
    out = np.empty(Z.size, np.float64)
    lib().orc_rhs_phi_water(Z.size, _dp(Z), _dp(vlow), _dp(vup), rho, g, _dp(out))
    return out


def rhs_phi_helium(Z, vlow, h: float, vdw: float) -> np.ndarray:
    Z, vlow = _c128(Z), _c128(vlow)
    out = np.empty(Z.size, np.float64)
    lib().orc_rhs_phi_helium(Z.size, _dp(Z), _dp(vlow), h, vdw, _dp(out))
    return out


def rhs(problem: Problem, x, y, phi, diagnostics: bool = False):
    """One RHS evaluation: returns (dx, dy, dphi[, a, zp, zpp]) and the LU info."""
    x, y, phi = _f64(x), _f64(y), _f64(phi)
    n = x.size
    dx, dy, dphi, a = (np.empty(n) for _ in range(4))
    zp = np.empty(n, np.complex128)
    zpp = np.empty(n, np.complex128)
    cp = problem.to_c()
    info = lib().orc_rhs(ctypes.byref(cp), n, _dp(x), _dp(y), _dp(phi), _dp(dx), _dp(dy), _dp(dphi),
                         _dp(a), _dp(zp), _dp(zpp))
    if diagnostics:
        return (dx, dy, dphi, a, zp, zpp), info
    return (dx, dy, dphi), info


def rk4_steps(problem: Problem, x, y, phi, dt: float, steps: int):
    x, y, phi = _f64(x).copy(), _f64(y).copy(), _f64(phi).copy()
    cp = problem.to_c()
    info = lib().orc_rk4_steps(ctypes.byref(cp), x.size, float(dt), int(steps), _dp(x), _dp(y), _dp(phi))
    return (x, y, phi), info


def rhs_driven(problem: Problem, drive: Drive, x, y, phi, dl=None):
    """Driven helium RHS: (dx, dy, dphi[, dD]) and the LU info."""
    x, y, phi = _f64(x), _f64(y), _f64(phi)
    n = x.size
    dl = _f64(dl if dl is not None else np.zeros(n))
    dx, dy, dphi, ddl = (np.empty(n) for _ in range(4))
    cp, cd = problem.to_c(), drive.to_c()
    info = lib().orc_rhs_driven(ctypes.byref(cp), ctypes.byref(cd), n, _dp(x), _dp(y), _dp(phi), _dp(dl),
                                _dp(dx), _dp(dy), _dp(dphi), _dp(ddl))
    out = (dx, dy, dphi, ddl) if drive.augmented else (dx, dy, dphi)
    return out, info


def rk4_steps_driven(problem: Problem, drive: Drive, x, y, phi, dl, dt: float, steps: int):
    x, y, phi = _f64(x).copy(), _f64(y).copy(), _f64(phi).copy()
    dl = _f64(dl if dl is not None else np.zeros(x.size)).copy()
    cp, cd = problem.to_c(), drive.to_c()
    info = lib().orc_rk4_steps_driven(ctypes.byref(cp), ctypes.byref(cd), x.size, float(dt), int(steps),
                                      _dp(x), _dp(y), _dp(phi), _dp(dl))
    return (x, y, phi, dl), info


def rkf45_evolve(problem: Problem, x, y, phi, t0: float, t1: float, atol: float = 1e-6, rtol: float = 1e-3,
                 h_min: float = 1e-16, h_max: float = 1e10, h0: float = 1e-2, max_rejected: int = 500,
                 max_times: int = 100000):
    """Adaptive RKF45 (orc_rkf45_evolve): returns ((x, y, phi), status, t, h, accepted, rejected, times)."""
    x, y, phi = _f64(x).copy(), _f64(y).copy(), _f64(phi).copy()
    cp = problem.to_c()
    t, h = ctypes.c_double(), ctypes.c_double()
    acc, rej = ctypes.c_longlong(), ctypes.c_longlong()
    times = np.zeros(max_times)
    st = lib().orc_rkf45_evolve(ctypes.byref(cp), x.size, t0, t1, atol, rtol, h_min, h_max, h0, max_rejected,
                                _dp(x), _dp(y), _dp(phi), ctypes.byref(t), ctypes.byref(h), ctypes.byref(acc),
                                ctypes.byref(rej), _dp(times), max_times)
    return (x, y, phi), st, t.value, h.value, acc.value, rej.value, times[:min(acc.value, max_times)]


def invariants(problem: Problem, x, y, phi, u, v, kappa: float = 0.0) -> np.ndarray:
    x, y, phi, u, v = _f64(x), _f64(y), _f64(phi), _f64(u), _f64(v)
    out = np.empty(5)
    cp = problem.to_c()
    lib().orc_invariants(ctypes.byref(cp), x.size, _dp(x), _dp(y), _dp(phi), _dp(u), _dp(v), kappa, _dp(out))
    return out


# ------------------------------------------------------------------ implicit GL2
# Two-stage Gauss-Legendre (order 4) with damped Newton, as GaussLegendre2
# (GaussLegendre.cuh:216-605, GLCoefficients.hpp:5-17, JacobianCalculator.cuh:223-284).
# Generic over the right-hand side f: R^m -> R^m.  The Newton matrix is the
# exact one of the stage equations R_i = k_i - f(y + h sum_j A_ij k_j):
#   dR_i/dk_j = delta_ij I - h A_ij J(y_i);
# the residual norm runs over both stages; the Armijo target stays at the
# iteration's base point (phi(k + a d) <= phi(k) - c a |R(k)|^2); the step is
# halved up to max_halvings times down to hmin = |t1 - t0| / 2^20 and then kept.
_SQ3 = 1.7320508075688772935
GL2_A = ((0.25, 0.25 - _SQ3 / 6.0), (0.25 + _SQ3 / 6.0, 0.25))
GL2_B = (0.5, 0.5)


def fd_jacobian(f, y, eps: float = 1e-6) -> np.ndarray:
    """Central differences, column j = (f(y + eps e_j) - f(y - eps e_j)) / (2 eps)."""
    y = _f64(y)
    m = y.size
    J = np.empty((m, m))
    for j in range(m):
        yp = y.copy()
        ym = y.copy()
        yp[j] += eps
        ym[j] -= eps
        J[:, j] = (f(yp) - f(ym)) / (2.0 * eps)
    return J


def perturbed_states(x, y, phi, eps: float) -> np.ndarray:
    """The 3N perturbed complex states of the batched finite-difference
    Jacobian (JacobianCalculator.cuh:11-75 createInitialBatchedZ, :154-161
    createInitialState): 6 N^2 complex values.  Perturbation b (b / N picks
    x, y or phi, b % N the node) has its positions Z = x + i y at [b N, (b+1) N)
    and its potentials phi + 0 i at [3 N^2 + b N, ...); the perturbed entry is
    the complex sum with (eps, 0) or (0, eps), both parts added."""
    x, y, phi = _f64(x), _f64(y), _f64(phi)
    n = x.size
    re = np.empty((2, 3 * n, n))
    im = np.empty((2, 3 * n, n))
    re[0], im[0] = x, y
    re[1], im[1] = phi, 0.0
    for b in range(3 * n):
        c, j = divmod(b, n)
        part = 1 if c == 2 else 0
        re[part, b, j] = re[part, b, j] + (0.0 if c == 1 else eps)
        im[part, b, j] = im[part, b, j] + (eps if c == 1 else 0.0)
    out = np.empty(re.size, dtype=np.complex128)  # assembled without arithmetic: signs of zeros kept
    out.real = re.reshape(-1)
    out.imag = im.reshape(-1)
    return out


def gl2_step(f, jac, y, h: float, tol: float = 1e-10, max_newton: int = 20, allow_simplified: bool = False,
             armijo_c: float = 1e-4, backtrack: float = 0.5, min_alpha: float = 1e-6):
    """One GL2 step of size h: returns (converged, y_next, iterations, residual norm)."""
    (a11, a12), (a21, a22) = GL2_A
    m = y.size
    fy = f(y)
    k = np.concatenate([fy, fy])

    def residual(kk):
        y1 = y + h * (a11 * kk[:m] + a12 * kk[m:])
        y2 = y + h * (a21 * kk[:m] + a22 * kk[m:])
        return np.concatenate([kk[:m] - f(y1), kk[m:] - f(y2)]), (y1, y2)

    R, ys = residual(k)
    frozen = None
    converged = False
    it = 0
    for it in range(max_newton):
        nr = float(np.linalg.norm(R))
        if nr <= tol * (1.0 + float(np.linalg.norm(k))):
            converged = True
            break
        J1, J2 = (frozen, frozen) if frozen is not None else (jac(ys[0]), jac(ys[1]))
        eye = np.eye(m)
        M = np.block([[eye - h * a11 * J1, -h * a12 * J1], [-h * a21 * J2, eye - h * a22 * J2]])
        d = np.linalg.solve(M, -R)
        phi = 0.5 * nr * nr
        alpha = 1.0
        while True:
            kt = k + alpha * d
            Rt, yst = residual(kt)
            if 0.5 * float(Rt @ Rt) <= phi - armijo_c * alpha * nr * nr:
                k, R, ys = kt, Rt, yst
                break
            alpha *= backtrack
            if alpha < min_alpha:
                if frozen is None and allow_simplified:
                    frozen = jac(y)
                    break
                return False, None, it, float(np.linalg.norm(Rt))
    y_next = y + h * (GL2_B[0] * k[:m] + GL2_B[1] * k[m:])
    return converged, y_next, it, float(np.linalg.norm(R))


def gl2_evolve(f, y0, t0: float, t1: float, step: float, jac=None, tol: float = 1e-10, max_newton: int = 20,
               allow_simplified: bool = False, armijo_c: float = 1e-4, backtrack: float = 0.5,
               min_alpha: float = 1e-6, max_halvings: int = 6, eps: float = 1e-6):
    """GaussLegendre2::runEvolution (GaussLegendre.cuh:227-330): returns (times, states), the
    initial point included; raises RuntimeError when a step fails at every halving."""
    if jac is None:
        jac = lambda yy: fd_jacobian(f, yy, eps)  # noqa: E731
    y = _f64(y0).copy()
    fwd = 1.0 if t1 >= t0 else -1.0
    hmin = abs(t1 - t0) / 2.0 ** 20
    t = t0
    times, states = [t], [y.copy()]
    while (t - t1) * fwd < 0.0:
        htry = min(step, abs(t1 - t)) * fwd
        ok = False
        for _ in range(max_halvings + 1):
            ok, yn, _, res = gl2_step(f, jac, y, htry, tol, max_newton, allow_simplified, armijo_c, backtrack,
                                      min_alpha)
            if ok or abs(htry) <= hmin:
                break
            htry *= 0.5
        if not ok:
            raise RuntimeError(f"GL2 failed to converge at t={t}; residual {res:.3e}; last h {htry:.3e}")
        y = yn
        t += htry
        step = abs(htry)
        times.append(t)
        states.append(y.copy())
    return np.array(times), np.array(states)


def boundary_rhs(problem: Problem):
    """The oracle RHS as f(state) on the real state [x | y | phi]."""
    def f(s):
        n = s.size // 3
        (dx, dy, dp), _ = rhs(problem, s[:n], s[n:2 * n], s[2 * n:])
        return np.concatenate([dx, dy, dp])
    return f
