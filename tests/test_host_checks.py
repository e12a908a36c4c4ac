"""Host-side argument checks of the Python mirror: wrong sizes are rejected
before any library call, so no export reads past the end of a host array.
The checks of Python/integration/rhs.py (equal lengths; 256 * batch_size for
the batched export) are kept, and the fixed-size exports also check their N."""
import numpy as np
import pytest

from superfluid_dynamics_gb300.engine import Engine, SimulationManager


class _NoCalls:
    """Stands in for the library: any call reaching it fails the test."""

    def __getattr__(self, name):
        def fail(*a, **k):
            raise AssertionError(f"{name} was called")
        return fail


def _manager():
    m = SimulationManager.__new__(SimulationManager)
    m.lib = _NoCalls()
    return m


def _engine(ntot):
    e = Engine.__new__(Engine)
    e._L = _NoCalls()
    e._h = None
    e.ntot = ntot
    return e


@pytest.mark.parametrize("fn, n", [("calculate_rhs256_from_vectors", 255), ("calculate_rhs256_from_vectors", 512),
                                   ("calculate_rhs2048_from_vectors", 2047)])
def test_fixed_size_exports_check_n(fn, n):
    v = np.zeros(n)
    with pytest.raises(ValueError, match="nodes"):
        getattr(_manager(), fn)(v, v, v, 1.0, 0.0, 0.0, 1.0)


def test_unequal_lengths_rejected():
    m = _manager()
    with pytest.raises(ValueError, match="same length"):
        m.calculate_rhs_from_vectors(np.zeros(64), np.zeros(64), np.zeros(63), 1.0, 0.0, 0.0, 1.0)
    with pytest.raises(ValueError, match="same length"):
        m.calculate_vorticities256_from_vectors(np.zeros(256, complex), np.zeros(255, complex), 1.0, 0.0, 0.0, 1.0)


@pytest.mark.parametrize("nx, ny, nphi, batch", [(512, 512, 256, 2), (511, 511, 512, 2), (512, 512, 512, 0),
                                                 (510, 512, 512, 2)])
def test_batched_export_checks_256_per_surface(nx, ny, nphi, batch):
    with pytest.raises(ValueError, match="256 \\* batch_size"):
        _manager().calculate_rhs256_from_vectors_batched(np.zeros(nx), np.zeros(ny), np.zeros(nphi), 1.0, 0.0, 0.0,
                                                         1.0, batch)


def test_derivative_export_checks_n():
    with pytest.raises(ValueError, match="256"):
        _manager().calculate_derivativeFFT256(np.zeros(128, complex))


def test_engine_state_arrays_checked():
    e = _engine(96)
    with pytest.raises(ValueError):
        e.set_state(np.zeros(96), np.zeros(96), np.zeros(95))
    with pytest.raises(ValueError):
        e.set_aux(np.zeros(95))
    x = np.zeros(96)
    with pytest.raises(ValueError):
        e.step_host(x, x, np.zeros(97), 0.01, 1)
    with pytest.raises(ValueError):
        e.step_host(x, x, np.zeros(96, np.float32), 0.01, 1)
    with pytest.raises(ValueError):  # step_host writes back in place: a strided view is refused
        e.step_host(x, x, np.zeros(192)[::2], 0.01, 1)


def test_manager_binds_a_library_loaded_from_a_path():
    """SimulationManager(dll_path) binds the export signatures like the default
    load, so float arguments pass and the error code comes back."""
    from superfluid_dynamics_gb300 import _lib
    path = _lib.load()._name
    m = SimulationManager(path)
    v = np.zeros(256)
    assert m.lib.calculatePerturbedStates256.argtypes is not None
    rc, Z = m.calculate_perturbed_states256(v, v, v, 1e-6, 145.0, 0.0, 1.5e-8, 1e-6)
    assert rc == 0 and Z[0] == 1e-6 + 0j


def test_reverse_mode_arrays_checked_before_device_work():
    """The Jacobian writes 9 (3 ntot)^2 values and the VJPs read 3 ntot: a
    state of another length is refused on the host, before any copy."""
    e = _engine(32)
    bad, good = np.zeros(95), np.zeros(96)
    with pytest.raises(ValueError, match="96"):
        e.jacobian(bad)
    with pytest.raises(ValueError, match="96"):
        e.rhs_vjp(good, bad)
    with pytest.raises(ValueError, match="96"):
        e.rk4_record(0.01, 1, 1, bad)
    with pytest.raises(ValueError, match="96"):
        e.rk4_vjp(bad)
