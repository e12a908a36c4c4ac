"""The reference's own ctypes binding (CuSuperHelium/Python/integration/rhs.py)
driving libsfd.so.

tests/golden/ref_rhs_bindings.json holds every argtypes / restype declaration
and every ctypes Structure of rhs.py, as written there (extracted with `ast` by
tests/golden/make_binding_spec.py; rhs.py itself imports only on Windows).

On the CPU:
  * every symbol rhs.py binds resolves in libsfd.so, except the export this
    library leaves out (integrateOptomechanicalSimulationRK4 and its free
    function, whose delayed-intensity update races in the reference);
  * rhs.py's Structures lay out like this library's structs (sizes, offsets);
  * where a reference checkout is present (SFD_REFERENCE_DIR), the fixture
    still matches rhs.py.
On the GPU, a CDLL of libsfd.so with rhs.py's declarations applied verbatim
is called the way rhs.py's SimulationManager calls it (structs by value, as
rhs.py declares them: on aarch64, the GB300 host, a composite above 16 bytes
travels by reference, which is what the C functions take), and every result
equals this package's SimulationManager bit for bit.
"""
import ctypes
import json
import os
import platform
from ctypes import POINTER, c_bool, c_char_p, c_double, c_int, c_size_t

import numpy as np
import pytest
from numpy.ctypeslib import ndpointer

import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import _lib
from superfluid_dynamics_gb300 import build as _build
from superfluid_dynamics_gb300 import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
SPEC = json.load(open(os.path.join(HERE, "golden", "ref_rhs_bindings.json")))
LEFT_OUT = {"integrateOptomechanicalSimulationRK4", "integrateOptomechanicalSimulationRK4_freeMemory"}
OURS = {"CSimulationProperties": _lib.SimProperties, "CGaussLegendreProperties": _lib.GaussLegendreOptions,
        "CRK4Options": _lib.RK4SolverOptions, "COptomechanicalProperties": _lib.COptomechanicalVariables}
_SIMPLE = {"c_double": c_double, "c_int": c_int, "c_size_t": c_size_t, "c_char_p": c_char_p, "c_bool": c_bool,
           "int": c_int, "complex128": np.complex128}


def _structures():
    out = {}
    for name, st in SPEC["structures"].items():
        out[name] = type(name, (ctypes.Structure,), {"_fields_": [(f, _SIMPLE[t]) for f, t in st["fields"]]})
    return out


STRUCTS = _structures()


def _ctype(d, by_value=True):
    if d["kind"] == "ndpointer":
        return ndpointer(_SIMPLE[d["dtype"]], flags=tuple(d["flags"]))
    if d["kind"] == "pointer":
        return POINTER(_ctype(d["to"]))
    name = d["name"]
    if name in STRUCTS:
        return STRUCTS[name] if by_value else POINTER(STRUCTS[name])
    return _SIMPLE[name]


def _ref_lib():
    """libsfd.so with rhs.py's declarations applied as written (on hosts
    other than aarch64 the by-value Structures become pointers)."""
    _lib.load()  # builds if needed
    lib = ctypes.CDLL(_build.LIB)
    by_value = platform.machine() in ("aarch64", "arm64")
    for sym, f in SPEC["functions"].items():
        if sym in LEFT_OUT:
            continue
        fn = getattr(lib, sym)
        fn.argtypes = tuple(_ctype(a, by_value) for a in f["argtypes"])
        fn.restype = _ctype(f["restype"])
    return lib, by_value


def test_every_bound_symbol_resolves():
    _lib.load()
    lib = ctypes.CDLL(_build.LIB)
    missing = [s for s in SPEC["functions"] if s not in LEFT_OUT and not hasattr(lib, s)]
    assert not missing, missing
    assert len(SPEC["functions"]) == 16 and LEFT_OUT <= set(SPEC["functions"])


def test_structures_lay_out_like_ours():
    for name, ours in OURS.items():
        ref = STRUCTS[name]
        assert ctypes.sizeof(ref) == ctypes.sizeof(ours), name
        for (fr, tr), (fo, to) in zip(ref._fields_, ours._fields_):
            assert getattr(ref, fr).offset == getattr(ours, fo).offset, (name, fr, fo)
            assert ctypes.sizeof(tr) == ctypes.sizeof(to), (name, fr)


def test_fixture_matches_the_reference_source():
    ref = os.environ.get("SFD_REFERENCE_DIR")
    path = os.path.join(ref or "", SPEC["source"])
    if not ref or not os.path.exists(path):
        pytest.skip("no reference checkout (SFD_REFERENCE_DIR)")
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_binding_spec", os.path.join(HERE, "golden", "make_binding_spec.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert mod.extract(path) == SPEC


def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _wave(n, seed=2):
    s = W.random_modes(n, seed=seed)
    return np.ascontiguousarray(s.x), np.ascontiguousarray(s.y), np.ascontiguousarray(s.phi)


def _same(a, b):
    return all(np.array_equal(u, v) for u, v in zip(a, b))


@pytest.mark.gpu
def test_rhs_and_transform_exports_through_the_reference_binding():
    _gpu()
    lib, _ = _ref_lib()
    ours = sfd.SimulationManager()
    L, rho, kappa, depth = 2 * np.pi, 0.0, 0.0, 1.0
    # calculateRHSFromVectors: called as rhs.py:117-135 calls it
    x, y, phi = _wave(128)
    vx, vy, dphi = np.empty_like(x), np.empty_like(x), np.empty_like(x)
    rc = lib.calculateRHSFromVectors(x, y, phi, vx, vy, dphi, L, rho, kappa, depth, len(x))
    r2 = ours.calculate_rhs_from_vectors(x, y, phi, L, rho, kappa, depth)
    assert rc == 0 == r2[0] and _same((vx, vy, dphi), r2[1:]) and np.isfinite(dphi).all()
    # calculateRHS256FromVectors (rhs.py:101-115) and the batched form (rhs.py:182-195)
    x, y, phi = _wave(256)
    vx, vy, dphi = np.empty_like(x), np.empty_like(x), np.empty_like(x)
    rc = lib.calculateRHS256FromVectors(x, y, phi, vx, vy, dphi, L, rho, kappa, depth)
    r2 = ours.calculate_rhs256_from_vectors(x, y, phi, L, rho, kappa, depth)
    assert rc == 0 == r2[0] and _same((vx, vy, dphi), r2[1:])
    xb, yb, pb = np.concatenate([x, x]), np.concatenate([y, y[::-1]]), np.concatenate([phi, phi[::-1]])
    vx, vy, dphi = np.empty_like(xb), np.empty_like(xb), np.empty_like(xb)
    rc = lib.calculateRHS256FromVectorsBatched(xb, yb, pb, vx, vy, dphi, L, rho, kappa, depth, 2)
    r2 = ours.calculate_rhs256_from_vectors_batched(xb, yb, pb, L, rho, kappa, depth, 2)
    assert rc == 0 == r2[0] and _same((vx, vy, dphi), r2[1:])
    # calculateVorticities256FromVectors (rhs.py:155-168) and calculateDerivativeFFT256 (rhs.py:170-180)
    Z = np.ascontiguousarray(x + 1j * y)
    P = np.ascontiguousarray(phi.astype(np.complex128))
    a, Zp, Zpp = np.empty(256), np.empty(256, np.complex128), np.empty(256, np.complex128)
    rc = lib.calculateVorticities256FromVectors(Z, P, a, Zp, Zpp, L, rho, kappa, depth)
    r2 = ours.calculate_vorticities256_from_vectors(Z, P, L, rho, kappa, depth)
    assert rc == 0 == r2[0] and _same((a, Zp, Zpp), r2[1:])
    out = np.empty(256, np.complex128)
    rc = lib.calculateDerivativeFFT256(Z, out)
    r2 = ours.calculate_derivativeFFT256(Z)
    assert rc == 0 == r2[0] and np.array_equal(out, r2[1])


@pytest.mark.gpu
def test_struct_exports_through_the_reference_binding():
    """GL2 integration (rhs.py:224-264), the augmented drive's RHS and RK4
    (rhs.py:306-358) and the Jacobian (rhs.py:213-222), each with rhs.py's
    Structures."""
    _gpu()
    lib, by_value = _ref_lib()
    ours = sfd.SimulationManager()
    wrap = (lambda s: s) if by_value else ctypes.byref
    n = 32
    x, y, phi = _wave(n)
    y0 = np.ascontiguousarray(np.concatenate([x, y, phi]))
    S = STRUCTS
    sp = S["CSimulationProperties"](2 * np.pi, 0.0, 0.0, 1.0, False, 1, False)
    gl = S["CGaussLegendreProperties"](0.0, 0.02, 0.01, 1e-10, 20, False, True, 1e-4, 0.5, 1e-4, 10)
    states, times = POINTER(c_double)(), POINTER(c_double)()
    ns, nt = c_size_t(), c_size_t()
    rc = lib.integrateSimulationGL2(y0, ctypes.byref(states), ctypes.byref(ns), ctypes.byref(times),
                                    ctypes.byref(nt), wrap(sp), wrap(gl), n)
    assert rc == 0
    got = np.ctypeslib.as_array(states, shape=(ns.value, 3 * n)).copy()
    T = np.ctypeslib.as_array(times, shape=(nt.value,)).copy()
    lib.integrateSimulationGL2_freeMemory(states, times)
    rc2, T2, S2 = ours.integrate(y0, _lib.SimProperties(2 * np.pi, 0.0, 0.0, 1.0, False, 1, False),
                                 _lib.GaussLegendreOptions(0.0, 0.02, 0.01, 1e-10, 20, False, True, 1e-4, 0.5, 1e-4,
                                                           10))
    assert rc2 == 0 and np.array_equal(T, T2) and np.array_equal(got, S2)
    # the augmented optomechanical drive: a 15 nm helium film of 1 um period
    # (SI properties, nondimensional state), drive terms strong enough to show
    L, depth, alpha = 1e-6, 15e-9, 3.5e-24
    Lb = L / (2 * np.pi)
    Tb = np.sqrt(Lb / (3 * alpha / depth ** 4))  # the reference's time unit (Export.cu:1222-1246)
    xi = W.nodes(n)
    state = np.ascontiguousarray(np.concatenate([xi, 0.05 * (depth / Lb) * np.cos(2 * xi), 0.001 * np.sin(xi),
                                                 1e-3 * np.cos(xi)]))
    props = (L, 150.0, 0.0, depth, False, 1, False)
    drive = (3e7, 5e7, 2e14, 1e-6, 1e9, 0.0, 5e-7, 1e-7, 1e3, 0.05)
    sph, opt = S["CSimulationProperties"](*props), S["COptomechanicalProperties"](*drive)
    rhs = np.empty_like(state)
    assert lib.calculateRhsAugmentedOptomechanical(state, rhs, wrap(sph), wrap(opt), n) == 0
    sp2, op2 = _lib.SimProperties(*props), _lib.COptomechanicalVariables(*drive)
    assert np.array_equal(rhs, ours.calculate_augmented_rhs(state, sp2, op2)) and np.isfinite(rhs).all()
    dt = 1e-3 * Tb
    ro = S["CRK4Options"](dt, 0.0, 3.5 * dt, True)
    states, times = POINTER(c_double)(), POINTER(c_double)()
    rc = lib.integrateAugmentedOptomechanicalSimulationRK4(state, ctypes.byref(states), ctypes.byref(ns),
                                                           ctypes.byref(times), ctypes.byref(nt), wrap(sph),
                                                           wrap(ro), wrap(opt), n)
    assert rc == 0
    got = np.ctypeslib.as_array(states, shape=(ns.value, 4 * n)).copy()
    lib.integrateAugmentedOptomechanicalSimulationRK4_freeMemory(states, times)
    rc2, _, S2 = ours.integrate_augmented_optomechanical_problem(state, sp2, op2,
                                                                 _lib.RK4SolverOptions(dt, 0.0, 3.5 * dt, True))
    assert rc2 == 0 and np.array_equal(got, S2) and got.shape[0] >= 2
    # the finite-difference Jacobian into a Fortran-ordered array
    J = np.empty((3 * n, 3 * n), order="F")
    assert lib.calculateJacobian(y0, J, 2 * np.pi, 0.0, 0.0, 1.0, 1e-6, n) == 0
    rc2, J2 = ours.calculate_jacobian(x, y, phi, 2 * np.pi, 0.0, 0.0, 1.0, 1e-6)
    assert rc2 == 0 and np.array_equal(J, J2)
