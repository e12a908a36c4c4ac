"""HDF5 state and trajectory files (superfluid_dynamics_gb300.h5io) in the
reference's layouts: the reader against the two libhdf5-written trajectory
files the reference ships (when present), the writer's dataset encoding
against theirs, and round trips of the state-file (SimulationRunner.cuh:99-178)
and simulation-file (Python/simulation.py:97-130) layouts."""
import os
import struct

import numpy as np
import pytest

from superfluid_dynamics_gb300 import h5io

# the reference checkout, when this machine has one (SFD_REFERENCE_DIR)
_REF = os.path.join(os.environ.get("SFD_REFERENCE_DIR", ""), "CuSuperHelium", "Python")
_FILES = [os.path.join(_REF, "integration", "simulation_15modes.h5"),
          os.path.join(_REF, "simulation_gaussian_highampl0.1.h5")]


def _ref_file(i):
    if not os.path.exists(_FILES[i]):
        pytest.skip("reference trajectory files not present")
    return _FILES[i]


@pytest.mark.parametrize("i", [0, 1])
def test_reader_reads_the_reference_trajectories(i):
    ds, attrs = h5io.read(_ref_file(i))
    n = ds["x0"].size
    assert ds["Y"].shape == (ds["T"].size, 3 * n)
    assert np.all(np.diff(ds["T"]) > 0) and ds["T"][0] == 0.0
    # the first stored state is the initial state written beside it
    assert np.array_equal(ds["Y"][0], np.concatenate([ds["x0"], ds["y0"], ds["pot0"]]))


def _dataset_messages(path):
    b = open(path, "rb").read()
    R = h5io._Reader(b)
    bt = hp = None
    for t, body, _ in R.messages(R.u("Q", 64)[0]):
        if t == 0x11:
            bt, hp = struct.unpack_from("<QQ", body)
    hdata = R.u("Q", hp + 24)[0]
    snod = R.u("Q", bt + 32)[0]
    name = lambda off: b[hdata + off:b.index(b"\0", hdata + off)].decode()  # noqa: E731
    out = {}
    for i in range(R.u("H", snod + 6)[0]):
        off, oh = R.u("QQ", snod + 8 + 40 * i)
        # the layout message without its data address
        out[name(off)] = [(t, fl, body[:2] + body[10:18] if t == 0x8 else body)
                          for t, body, fl in R.messages(oh) if t != 0]
    keys = [name(R.u("Q", bt + 24)[0]), name(R.u("Q", bt + 40)[0])]
    return b[8:24], keys, list(out), out


def test_writer_encodes_datasets_as_libhdf5_does(tmp_path):
    ref = _ref_file(1)
    ds, _ = h5io.read(ref)
    mine = str(tmp_path / "t.h5")
    h5io.write(mine, {k: ds[k] for k in ("T", "Y", "x0", "y0", "pot0")})
    sb_a, keys_a, order_a, msgs_a = _dataset_messages(ref)
    sb_b, keys_b, order_b, msgs_b = _dataset_messages(mine)
    assert sb_a == sb_b and keys_a == keys_b and order_a == order_b
    assert msgs_a == msgs_b


def test_attribute_message_layout():
    body = h5io._attr_msg("depth", 2.5)
    t, size, flags = struct.unpack_from("<HHB", body)
    assert t == 0xC and size == len(body) - 8 and size % 8 == 0
    ver, _, nlen, dlen, slen = struct.unpack_from("<BBHHH", body, 8)
    assert (ver, nlen, dlen, slen) == (1, 6, 20, 8)
    assert body[16:22] == b"depth\0"
    value = struct.unpack_from("<d", body, 8 + 8 + 8 + 24 + 8)[0]
    assert value == 2.5


def test_state_file_round_trip_and_checks(tmp_path):
    n = 64
    xi = 2 * np.pi * np.arange(n) / n
    Z = xi + 1j * 0.05 * np.cos(xi)
    phi = 0.01 * np.sin(xi)
    p = str(tmp_path / "state.h5")
    props = {"rho": 0.3, "kappa": 1e-4, "U": 0.0, "depth": 2.0, "initial_amplitude": 0.05}
    assert h5io.save_state_file(p, Z, phi, props, rhs=True) == 0
    ds, attrs = h5io.read(p)
    assert ds["interface"].shape == (n, 2) and ds["potential"].shape == (n,)
    assert attrs == {**props, "rhs": True}
    Z2, phi2 = h5io.load_state_file(p, n, scale_y=2.0)
    assert np.array_equal(Z2.real, Z.real) and np.array_equal(Z2.imag, 2.0 * Z.imag)
    assert np.array_equal(phi2, phi)
    with pytest.raises(RuntimeError, match=r"Interface must have shape \(32, 2\), instead it has \(64, 2\)"):
        h5io.load_state_file(p, 32)


def test_simulation_file_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    n = 16
    T = np.linspace(0.0, 1.0, 11)
    Y = rng.normal(size=(11, 3 * n))
    p = str(tmp_path / "sim.h5")
    h5io.save_simulation_file(p, T, Y, Y[0], L=1e-3, depth=2e-8, t0=0.0, t1=1.0, initial_amplitude=1e-9, g=9.81)
    out = h5io.load_simulation_file(p)
    T2, Y2, Y02, L, depth, N, t0, t1, amp, g = out
    assert np.array_equal(T2, T) and np.array_equal(Y2, Y) and np.array_equal(Y02, Y[0])
    assert (L, depth, N, t0, t1, amp, g) == (1e-3, 2e-8, n, 0.0, 1.0, 1e-9, 9.81)
    assert isinstance(N, int)
    assert h5io.load_simulation_file(str(tmp_path / "missing.h5")) is None


def test_truncated_dataset_is_rejected(tmp_path):
    """A dataset whose data would run past the end of the file is a format
    error, found before the array is allocated (Python and C++ readers)."""
    import subprocess
    n = 16
    p = str(tmp_path / "state.h5")
    h5io.save_state_file(p, np.arange(n) + 0.5j, np.ones(n), {"depth": 1.0})
    raw = open(p, "rb").read()
    cut = str(tmp_path / "cut.h5")
    open(cut, "wb").write(raw[:-8])  # the last dataset's data ends the file
    with pytest.raises(h5io.H5FormatError, match="past the end"):
        h5io.read(cut)
    exe = _cxx_tool(tmp_path)
    bad = subprocess.run([exe, "read", cut, str(n)], capture_output=True, text=True)
    assert bad.returncode == 1 and "past the end" in bad.stderr


def test_not_hdf5_is_rejected(tmp_path):
    p = tmp_path / "x.h5"
    p.write_bytes(b"not an hdf5 file at all")
    with pytest.raises(h5io.H5FormatError):
        h5io.read(str(p))


# ---------------------------------------------------------------- C++ side (include/sfd_h5.hpp)
def _cxx_tool(tmp_path):
    import shutil
    import subprocess
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "h5_check")
    subprocess.check_call([cxx, "-std=c++17", "-O1", os.path.join(root, "tests", "cpp", "h5_check.cpp"),
                           "-I", os.path.join(root, "include"), "-o", exe])
    return exe


def test_cpp_and_python_writers_produce_the_same_bytes(tmp_path):
    import subprocess
    exe = _cxx_tool(tmp_path)
    pc = str(tmp_path / "cxx.h5")
    subprocess.check_call([exe, "write", pc])
    n = 8
    j = np.arange(n)
    Z = 0.25 * j + 1j * (0.5 * j - 1.0)
    pp = str(tmp_path / "py.h5")
    h5io.save_state_file(pp, Z, 0.1 * j, {"rho": 0.25, "kappa": 1e-3, "U": 0.0, "depth": 2.0,
                                          "initial_amplitude": 0.05}, rhs=True)
    assert open(pc, "rb").read() == open(pp, "rb").read()
    Zc, phic = h5io.load_state_file(pc, n)
    assert np.array_equal(Zc, Z) and np.array_equal(phic, 0.1 * j)


def test_cpp_reader_reads_python_files_and_checks_shapes(tmp_path):
    import subprocess
    exe = _cxx_tool(tmp_path)
    rng = np.random.default_rng(9)
    n = 12
    Z = rng.normal(size=n) + 1j * rng.normal(size=n)
    phi = rng.normal(size=n)
    p = str(tmp_path / "s.h5")
    h5io.save_state_file(p, Z, phi, {"depth": 3.0})
    out = subprocess.run([exe, "read", p, str(n)], capture_output=True, text=True, check=True).stdout
    vals = np.array([[float(v) for v in line.split()] for line in out.strip().splitlines()])
    assert np.array_equal(vals[:, 0], Z.real) and np.array_equal(vals[:, 1], Z.imag) and np.array_equal(vals[:, 2], phi)
    bad = subprocess.run([exe, "read", p, "5"], capture_output=True, text=True)
    assert bad.returncode == 1 and "Interface must have shape (5, 2), instead it has (12, 2)" in bad.stderr


@pytest.mark.parametrize("i", [0, 1])
def test_cpp_reader_reads_the_reference_trajectories(tmp_path, i):
    import subprocess
    path = _ref_file(i)
    exe = _cxx_tool(tmp_path)
    r = subprocess.run([exe, "traj", path], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr


def test_truncated_files_fail_cleanly(tmp_path):
    """Every truncation of a valid state file is refused with a format error:
    the Python reader raises H5FormatError, the C++ reader exits with status 1
    (a crash would be a negative status), and neither reads past the end."""
    import subprocess
    n = 8
    p = str(tmp_path / "state.h5")
    h5io.save_state_file(p, np.arange(n) + 0.25j, np.ones(n), {"depth": 2.0, "rho": 0.5})
    raw = open(p, "rb").read()
    exe = _cxx_tool(tmp_path)
    cut = str(tmp_path / "cut.h5")
    cuts = sorted(set(list(range(0, 128, 7)) + list(range(128, len(raw), max(1, len(raw) // 40))) + [len(raw) - 1]))
    for k in cuts:
        open(cut, "wb").write(raw[:k])
        with pytest.raises(h5io.H5FormatError):
            h5io.load_state_file(cut, n)
        r = subprocess.run([exe, "read", cut, str(n)], capture_output=True, text=True)
        assert r.returncode == 1, (k, r.returncode, r.stderr)


def test_corrupted_files_never_crash(tmp_path):
    """Seeded random byte corruptions of a state file: the C++ reader either
    reads it or exits with status 1 (never a signal, never a hang), and the
    Python reader returns or raises a format or shape error."""
    import subprocess
    n = 8
    p = str(tmp_path / "state.h5")
    h5io.save_state_file(p, np.arange(n) + 0.25j, np.ones(n), {"depth": 2.0, "rho": 0.5})
    raw = open(p, "rb").read()
    exe = _cxx_tool(tmp_path)
    rng = np.random.default_rng(5)
    bad = str(tmp_path / "bad.h5")
    for _ in range(150):
        b = bytearray(raw)
        for _ in range(int(rng.integers(1, 4))):
            b[int(rng.integers(0, len(b)))] = int(rng.integers(0, 256))
        open(bad, "wb").write(b)
        r = subprocess.run([exe, "read", bad, str(n)], capture_output=True, timeout=20)
        assert r.returncode in (0, 1), r.returncode
        try:
            h5io.load_state_file(bad, n)
        except (h5io.H5FormatError, RuntimeError):
            pass
