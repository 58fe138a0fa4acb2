"""sgmd: GB300-native implementation of the SurfaceGrowthConsole timestep path.

The compute runs in libsgmd.so (hand-written sm_103a CUDA kernels behind a C ABI, see
include/sg_api.h); this package is the Python face of that ABI.  Importing it does not load the
library; the first call that needs it does, and fails loudly if it has not been built.
"""
from ._lib import MODE_MIXED, MODE_PLAIN, SgError, SimParams, lib
from .engine import (Simulation, build_workload, default_input, init_coords, init_vels, read_input_file,
                     set_params)

__all__ = ["Simulation", "SimParams", "SgError", "MODE_PLAIN", "MODE_MIXED", "build_workload", "default_input",
           "init_coords", "init_vels", "read_input_file", "set_params", "lib"]
