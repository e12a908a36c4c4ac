"""The allocation-free RHS entry point (sfd_rhs_device_noalloc).

Some callers of this library cannot call cudaMalloc: code that runs inside
another framework's memory pool, a real-time loop that must not allocate once
it is running, or a host that forbids runtime device allocation.  For them the
library offers one RHS evaluation whose scratch lives in a static device array
of fixed size (surfaces of up to 1024 nodes).  These tests call it through the
C ABI several times in a row, on surfaces whose padded size grows and shrinks
between calls (water 1024, helium 96, water 1024 again), on a prime node count
(97, the generic odd-radix transform) and on the single-node lower bound, and
check each result against the engine's sfd_rhs_device on an FP64 engine,
within the FP64 tolerance used by the other parity tests.  They also check
that a surface above the limit is refused with a clear error, that a
non-finite input shows as non-finite output (the call reports no status
words), and, in a fresh process, that the call works when it is the first
call into the library (its first call on a device resolves the scratch
address).  The file name sorts last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import _lib
from superfluid_dynamics_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-11  # FP64 parity tolerance of tests/test_gpu_parity.py
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    return torch


def _existing_rhs(torch, n, phys, state):
    out = torch.empty(3 * n, dtype=torch.float64, device="cuda")
    with sfd.Engine(n, phys, sfd.Options(precision=sfd.PRECISION_FP64, use_graphs=False)) as e:
        e.rhs_device(state.data_ptr(), out.data_ptr())
        e.synchronize()
    return out.cpu().numpy()


def _noalloc(torch, L, n, phys, state):
    out = torch.full((3 * n,), float("nan"), dtype=torch.float64, device="cuda")
    prob = phys.to_c()
    stream = torch.cuda.current_stream()
    rc = L.sfd_rhs_device_noalloc(ctypes.byref(prob), n, ctypes.c_void_p(state.data_ptr()),
                                  ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, L.sfd_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _helium96():
    xi = W.nodes(96)
    return W.Surface(xi.copy(), 0.4 * np.cos(2 * xi), 0.01 * np.sin(xi))


def _water(n, seed):
    xi = W.nodes(n)
    rng = np.random.default_rng(seed)
    y = sum(0.02 / m * rng.uniform() * np.cos(m * xi + rng.uniform(0, 2 * np.pi)) for m in range(1, 5))
    return W.Surface(xi.copy(), y, 0.5 * y[::-1].copy())


def test_noalloc_rhs_matches_engine_on_calls_in_a_row():
    torch = _torch()
    L = _lib.load()
    cases = [
        (1024, sfd.WaterBoundaryProblem(), W.random_modes(1024, seed=2)),
        (96, sfd.HeliumBoundaryProblem(8.0, 900.0), _helium96()),
        (1024, sfd.WaterBoundaryProblem(), W.random_modes(1024, seed=5)),
        (97, sfd.WaterBoundaryProblem(), _water(97, 7)),
        (1, sfd.WaterBoundaryProblem(), W.Surface(np.zeros(1), np.array([0.01]), np.array([0.002]))),
    ]
    for n, phys, s in cases:
        state = torch.tensor(np.concatenate([s.x, s.y, s.phi]), dtype=torch.float64, device="cuda")
        got = _noalloc(torch, L, n, phys, state)
        ref = _existing_rhs(torch, n, phys, state)
        assert np.isfinite(got).all(), n
        assert _rel(got[:2 * n], ref[:2 * n]) < TOL, n
        assert _rel(got[2 * n:], ref[2 * n:]) < TOL, n


def test_noalloc_nonfinite_input_gives_nonfinite_output():
    torch = _torch()
    L = _lib.load()
    s = W.random_modes(128, seed=2)
    y = s.y.copy()
    y[9] = np.nan
    state = torch.tensor(np.concatenate([s.x, y, s.phi]), dtype=torch.float64, device="cuda")
    got = _noalloc(torch, L, 128, sfd.WaterBoundaryProblem(), state)
    assert not np.isfinite(got).all()


def test_noalloc_rejects_oversized_surface():
    torch = _torch()
    L = _lib.load()
    prob = sfd.WaterBoundaryProblem().to_c()
    buf = torch.zeros(3 * 2048, dtype=torch.float64, device="cuda")
    rc = L.sfd_rhs_device_noalloc(ctypes.byref(prob), 2048, ctypes.c_void_p(buf.data_ptr()),
                                  ctypes.c_void_p(buf.data_ptr()), None)
    assert rc == -1
    assert b"1024" in L.sfd_last_error()


_FIRST_CALL = r"""
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import _lib
from superfluid_dynamics_gb300 import workloads as W
n = 256
s = W.random_modes(n, seed=3)
state = torch.tensor(np.concatenate([s.x, s.y, s.phi]), dtype=torch.float64, device="cuda")
out = torch.empty(3 * n, dtype=torch.float64, device="cuda")
L = _lib.load()
prob = sfd.WaterBoundaryProblem().to_c()
rc = L.sfd_rhs_device_noalloc(ctypes.byref(prob), n, ctypes.c_void_p(state.data_ptr()),
                              ctypes.c_void_p(out.data_ptr()), None)
assert rc == 0, L.sfd_last_error()
torch.cuda.synchronize()
got = out.cpu().numpy()
ref = torch.empty(3 * n, dtype=torch.float64, device="cuda")
with sfd.Engine(n, sfd.WaterBoundaryProblem(), sfd.Options(precision=sfd.PRECISION_FP64, use_graphs=False)) as e:
    e.rhs_device(state.data_ptr(), ref.data_ptr())
    e.synchronize()
ref = ref.cpu().numpy()
print("rel", float(np.abs(got - ref).max() / np.abs(ref).max()))
"""


def test_noalloc_as_first_library_call_in_a_fresh_process():
    """A new process whose first call into libsfd.so is the allocation-free
    entry point (its device buffers come from torch, so CUDA itself is already
    initialised): the per-device set-up of that first call runs there."""
    _torch()
    out = subprocess.run([sys.executable, "-c", _FIRST_CALL, ROOT], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    rel = float(out.stdout.split("rel")[-1])
    assert rel < TOL
