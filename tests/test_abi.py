"""CPU tests of the boundary: the C-ABI library builds for sm_103a, loads and
exports every function include/sfd.h declares; calls that need no GPU behave."""
import ctypes
import os

import pytest

from superfluid_dynamics_gb300 import _lib, build


def test_library_builds_and_exports_every_header_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    names = _lib.header_symbols()
    assert "sfd_create" in names and "calculateRHSFromVectors" in names and "integrateSimulationRK4" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"
    # every bound signature is a header symbol
    assert set(_lib._SIGS) <= set(names)


def test_version_and_defaults_without_gpu():
    L = _lib.load()
    assert b"sm_103a" in L.sfd_version()
    o = _lib.SfdOptions()
    L.sfd_default_options(ctypes.byref(o))
    assert o.precision == _lib.PRECISION_MIXED and o.refine_iters >= 1
    # the refinement fields sit after refactor_lag, past 4 bytes of padding
    assert o.extra_iters == 2 and o.refine_tol == 1e-10 and ctypes.sizeof(_lib.SfdOptions) == 56
    p = _lib.SfdProblem()
    L.sfd_default_problem(ctypes.byref(p))
    assert p.physics == _lib.WATER and p.gravity == 1.0
    assert L.sfd_set_default_precision(7) == -1
    assert b"precision" in L.sfd_last_error()


def test_struct_layouts_match_reference_exports():
    # ExportTypes.cuh:8-40 field order / sizes as bound by the reference's rhs.py
    assert ctypes.sizeof(_lib.SimProperties) == 48
    assert ctypes.sizeof(_lib.RK4SolverOptions) == 32


def test_create_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = _lib.load()
    n = (ctypes.c_int * 1)(64)
    p = _lib.SfdProblem()
    L.sfd_default_problem(ctypes.byref(p))
    h = ctypes.c_void_p()
    rc = L.sfd_create(n, 1, ctypes.byref(p), 1, None, ctypes.byref(h))
    assert rc == -4 and not h.value


def _build_facade_check(tmp_path):
    """Compile tests/cpp/facade_check.cpp against include/sfd.hpp and libsfd.so
    with the host C++ compiler (the facade is header-only C++17)."""
    import shutil
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib = _lib.load()  # builds libsfd.so if needed
    libdir = os.path.dirname(lib._name)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / "facade_check")
    cmd = [cxx, "-std=c++17", "-O1", os.path.join(root, "tests", "cpp", "facade_check.cpp"),
           "-I", os.path.join(root, "include"), "-I", os.path.join(cuda, "include"),
           "-L", libdir, "-lsfd", f"-Wl,-rpath,{libdir}",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-o", exe]
    subprocess.check_call(cmd)
    return exe


def test_cpp_facade_compiles_and_links(tmp_path):
    assert os.path.exists(_build_facade_check(tmp_path))


def test_c_caller_compiles_links_and_runs(tmp_path):
    """include/sfd.h is a C header: a C11 program (-pedantic) compiles against
    it, links to libsfd.so and gets the documented defaults and error codes
    without a device."""
    import shutil
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = _lib.load()
    libdir = os.path.dirname(lib._name)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / "abi_check")
    subprocess.check_call([cc, "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror",
                           os.path.join(root, "tests", "c", "abi_check.c"), "-I", os.path.join(root, "include"),
                           "-L", libdir, "-lsfd", f"-Wl,-rpath,{libdir}",
                           f"-Wl,-rpath-link,{os.path.join(cuda, 'lib64')}", "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
