"""The allocation-free RHS entry point (sfd_rhs_device_noalloc).

Some callers of this library cannot call cudaMalloc: code that runs inside
another framework's memory pool, a real-time loop that must not allocate once
it is running, or a host that forbids runtime device allocation.  For them the
library offers one RHS evaluation whose scratch lives in a static device array
of fixed size (surfaces of up to 1024 nodes).  This test calls it through the C
ABI twice in a row, each time on a different surface, and checks each result
against the engine's sfd_rhs_device on an FP64 engine, within the FP64
tolerance used by the other parity tests.  It also checks that a surface above
the limit is refused with a clear error.  The file name sorts last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import _lib
from superfluid_dynamics_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-11  # FP64 parity tolerance of tests/test_gpu_parity.py


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _existing_rhs(torch, n, phys, state):
    out = torch.empty(3 * n, dtype=torch.float64, device="cuda")
    with sfd.Engine(n, phys, sfd.Options(precision=sfd.PRECISION_FP64, use_graphs=False)) as e:
        e.rhs_device(state.data_ptr(), out.data_ptr())
        e.synchronize()
    return out.cpu().numpy()


def test_noalloc_rhs_matches_engine_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = _lib.load()
    cases = [
        (1024, sfd.WaterBoundaryProblem(), W.random_modes(1024, seed=2)),
        (96, sfd.HeliumBoundaryProblem(8.0, 900.0),
         W.Surface(W.nodes(96), 0.4 * np.cos(2 * W.nodes(96)), 0.01 * np.sin(W.nodes(96)))),
    ]
    stream = torch.cuda.current_stream()
    for n, phys, s in cases:
        state = torch.tensor(np.concatenate([s.x, s.y, s.phi]), dtype=torch.float64, device="cuda")
        out = torch.full((3 * n,), float("nan"), dtype=torch.float64, device="cuda")
        prob = phys.to_c()
        rc = L.sfd_rhs_device_noalloc(ctypes.byref(prob), n, ctypes.c_void_p(state.data_ptr()),
                                      ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.sfd_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        ref = _existing_rhs(torch, n, phys, state)
        assert np.isfinite(got).all()
        assert _rel(got[:2 * n], ref[:2 * n]) < TOL
        assert _rel(got[2 * n:], ref[2 * n:]) < TOL


def test_noalloc_rejects_oversized_surface():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = _lib.load()
    prob = sfd.WaterBoundaryProblem().to_c()
    buf = torch.zeros(3 * 2048, dtype=torch.float64, device="cuda")
    rc = L.sfd_rhs_device_noalloc(ctypes.byref(prob), 2048, ctypes.c_void_p(buf.data_ptr()),
                                  ctypes.c_void_p(buf.data_ptr()), None)
    assert rc == -1
    assert b"1024" in L.sfd_last_error()
