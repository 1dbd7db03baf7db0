"""astronomix_gb300 -- GB300-native MHD step with astronomix's API.

Drop-in for the accelerated path of leo1200/astronomix: the same
configuration objects, variable registry and ``time_integration`` entry
point, with the finite-volume (Pang-Wu split) and finite-difference (WENO-CT)
MHD steps running as hand-written sm_103a CUDA kernels behind the C ABI of
include/amx.h.
"""

from .option_classes import (
    SimulationConfig, SimulationParams, SnapshotSettings, BoundarySettings, BoundarySettings1D,
    finalize_config,
    FINITE_VOLUME, FINITE_DIFFERENCE, FORWARDS, BACKWARDS,
    MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA, VAN_ALBADA_PP,
    HLL, HLLC, HLLC_LM, LAX_FRIEDRICHS, HYBRID_HLLC, AM_HLLC,
    UNSPLIT, SPLIT, RK2_SSP, MUSCL, RK4_SSP,
    OPEN_BOUNDARY, REFLECTIVE_BOUNDARY, PERIODIC_BOUNDARY, MHD_JET_BOUNDARY,
    CARTESIAN, CYLINDRICAL, SPHERICAL,
    GHOST_CELLS, PERIODIC_ROLL, IMPLICIT_MIDPOINT, IMPLICIT_EULER,
    SINGLE_PRECISION, DOUBLE_PRECISION, WindParams,
    SIMPLE_SOURCE_TERM, DONOR_ACCOUNTING, RIEMANN_SPLIT, RIEMANN_SPLIT_UNSTABLE, HALF_SPLIT,
)
from .variable_registry import get_registered_variables, RegisteredVariables, StaticIntVector
from .setup_helpers import get_helper_data, construct_primitive_state, initialize_interface_fields, HelperData
from .time_integration import time_integration, gravitational_potential, SnapshotData, StateStruct

__version__ = "0.1.0"
