"""The C++ facade (include/sfd.hpp) run on the GPU: a compiled client program
checks BaseBoundaryIntegralCalculator::run, calculateVorticities, the
AutonomousRungeKuttaStepper and MatrixSolver against the engine's C ABI and a
host LU solve (tests/cpp/facade_check.cpp)."""
import subprocess

import pytest

from test_abi import _build_facade_check

pytestmark = pytest.mark.gpu


def test_cpp_facade_matches_c_abi(tmp_path):
    exe = _build_facade_check(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
