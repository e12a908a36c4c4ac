"""GB300-native Roberts-1983 boundary-integral engine (drop-in for the
CuSuperHelium RHS / RK4 path).  The compute lives in libsfd.so (CUDA, sm_103a)
behind the C ABI of include/sfd.h; this package is the Python host side."""
from ._lib import (HELIUM, PRECISION_FP64, PRECISION_MIXED, WATER, SfdError,  # noqa: F401
                   load as load_library)
from .engine import (AutonomousRungeKuttaStepper, BoundaryIntegralCalculator, Drive, Engine,  # noqa: F401
                     HeliumBoundaryProblem, Options, Physics, SimulationManager, WaterBoundaryProblem)
from . import h5io  # noqa: F401  (state / trajectory files in the reference's HDF5 layouts)

__all__ = ["Engine", "Options", "Physics", "Drive", "WaterBoundaryProblem", "HeliumBoundaryProblem",
           "BoundaryIntegralCalculator", "AutonomousRungeKuttaStepper", "SimulationManager",
           "WATER", "HELIUM", "PRECISION_FP64", "PRECISION_MIXED", "SfdError", "load_library", "h5io"]
