"""The streamed preconditioner product against the register-pipelined one,
and the early operand requests made before a kernel's wait on its predecessor.

A single-surface mixed engine applies X through k_gemv_hs: rows streamed into
shared memory by bulk copies, the first ones requested before the wait on the
preceding kernel.  k_gemv_h, the register-pipelined product batches use, sums
each row in the same order (per lane the chunks lane + 32 t, even t into one
accumulator and odd t into the other, then the same warp reduction), so an
engine stepped with either gives the same bits; the early requests of the
product and of the FP32 boundary-sum pass change timing only.  The choice is
read from the environment once per process (SFD_GEMV_SPW=0: register product;
SFD_GEMV_PREFETCH=0, SFD_SUMS_PREFETCH=0: no early requests), so each variant
runs in its own process: 70 RK4 steps of the bench's solver settings
(preconditioner rebuilt every 50 steps on the side stream, switched in 8 steps
later) on a water surface, the final states compared bit for bit.  N = 4096
streams two rows per warp; N = 1000 one, with a row length that is not a
multiple of 256 entries.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RUN = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import superfluid_dynamics_gb300 as sfd
from superfluid_dynamics_gb300 import workloads as W
n = int(sys.argv[2])
s = W.random_modes(n, seed=2)
opts = sfd.Options(precision=sfd.PRECISION_MIXED, refactor_every=50, refactor_lag=8, pre_iters=2,
                   refine_iters=2, autotune=False)
with sfd.Engine(n, sfd.WaterBoundaryProblem(), opts) as e:
    e.set_state(s.x, s.y, s.phi)
    e.step(0.005, 70)
    x, y, phi = e.get_state()
np.save(sys.argv[3], np.concatenate([x, y, phi]))
"""

_VARIANTS = (
    ("streamed", {}),
    ("register", {"SFD_GEMV_SPW": "0"}),
    ("no_early_requests", {"SFD_GEMV_PREFETCH": "0", "SFD_SUMS_PREFETCH": "0"}),
)


@pytest.mark.parametrize("n", [4096, 1000])
def test_streamed_product_and_early_requests_keep_the_bits(n, tmp_path):
    pytest.importorskip("torch")
    out = {}
    for name, env in _VARIANTS:
        f = tmp_path / f"{name}.npy"
        r = subprocess.run([sys.executable, "-c", _RUN, ROOT, str(n), str(f)], env={**os.environ, **env},
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        out[name] = np.load(f)
    assert np.isfinite(out["streamed"]).all()
    for name in ("register", "no_early_requests"):
        diff = np.abs(out[name] - out["streamed"]).max()
        assert np.array_equal(out[name], out["streamed"]), f"{name}: max |difference| {diff:.3e}"
