"""Reference exports whose work is host-side (no GPU needed): the perturbed
states of the finite-difference Jacobian, bit for bit against the oracle's
restatement of JacobianCalculator.cuh:11-75, and the file checks of
calculateRHS256FromFile, which fail before any device work."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from superfluid_dynamics_gb300 import h5io
from superfluid_dynamics_gb300.engine import SimulationManager


@pytest.fixture(scope="module")
def mgr():
    return SimulationManager()


def test_perturbed_states_match_the_oracle_bit_for_bit(mgr):
    rng = np.random.default_rng(11)
    n = 256
    x, y, phi = rng.normal(size=n), rng.normal(size=n), rng.normal(size=n)
    y[3] = -0.0   # the reference adds (eps, 0) as a complex sum: -0.0 + 0.0 = +0.0
    phi[7] = -0.0
    for eps in (1e-6, 3.5e-3):
        rc, Z = mgr.calculate_perturbed_states256(x, y, phi, 1e-6, 145.0, 0.0, 1.5e-8, eps)
        ref = O.perturbed_states(x, y, phi, eps)
        assert rc == 0 and Z.shape == (6 * n * n,)
        assert np.array_equal(Z.view(np.uint64), ref.view(np.uint64))
    # spot checks of the layout: perturbation b = N + 3 raises y_3, b = 2N + 7 raises phi_7
    b = n + 3
    assert Z[b * n + 3] == complex(x[3], 0.0 + 3.5e-3)
    assert np.signbit(Z[3].imag)  # an unperturbed entry keeps y_3 = -0.0
    assert Z[3 * n * n + (2 * n + 7) * n + 7] == complex(3.5e-3, 0.0)


def test_perturbed_states_need_256_nodes(mgr):
    v = np.zeros(128)
    with pytest.raises(ValueError, match="256"):
        mgr.calculate_perturbed_states256(v, v, v, 1.0, 0.0, 0.0, 1.0)


def test_rhs_from_file_rejects_bad_files_before_device_work(mgr, tmp_path):
    missing = str(tmp_path / "missing.h5")
    out = str(tmp_path / "out.h5")
    assert mgr.calculate_rhs256(missing, out, 1e-6, 145.0, 0.0, 1.5e-8) == -1
    assert "missing.h5" in mgr.lib.sfd_last_error().decode()
    small = str(tmp_path / "small.h5")
    xi = 2 * np.pi * np.arange(128) / 128
    h5io.save_state_file(small, xi + 0.01j * np.cos(xi), np.zeros(128), {"depth": 1.0})
    assert mgr.calculate_rhs256(small, out, 1e-6, 145.0, 0.0, 1.5e-8) == -1
    assert "Interface must have shape (256, 2), instead it has (128, 2)" in mgr.lib.sfd_last_error().decode()
    short_phi = str(tmp_path / "short_phi.h5")
    xi = 2 * np.pi * np.arange(256) / 256
    h5io.write(short_phi, {"interface": np.stack([xi, 0.01 * np.cos(xi)], axis=1), "potential": np.zeros(200)})
    assert mgr.calculate_rhs256(short_phi, out, 1e-6, 145.0, 0.0, 1.5e-8) == -1
    assert "potential holds 200 values" in mgr.lib.sfd_last_error().decode()
    assert not os.path.exists(out)
