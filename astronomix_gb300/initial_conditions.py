"""Initial conditions of the reference's self-gravity test problem.

``evrard_collapse`` builds the state and configuration of Evrard's collapse
exactly as astronomix's tests/self_gravity_tests/simulate_collapse.py sets
it up, so that the self-gravity path can be run and measured on the
reference's own problem.
"""

import numpy as np

from .option_classes import (
    SimulationConfig, SimulationParams, BoundarySettings, BoundarySettings1D, REFLECTIVE_BOUNDARY, SPLIT, MUSCL,
    HLLC, MINMOD, RIEMANN_SPLIT_UNSTABLE, finalize_config,
)
from .variable_registry import get_registered_variables
from .setup_helpers import get_helper_data, construct_primitive_state


def evrard_collapse(n, dtype=np.float32, t_end=3.0, version=RIEMANN_SPLIT_UNSTABLE):
    """Evrard's collapse on n^3 cells: a gas sphere of mass 1 and radius 1
    with rho = 1 / (2 pi r) inside (1e-4 outside), specific internal energy
    0.05, at rest, in a reflective box of side 4 (so the Poisson solve is the
    open-boundary one); split MUSCL-Hancock, HLLC, MINMOD, the given
    self-gravity version, C_cfl 0.4, G = 1, gamma 5/3.  Returns
    (config, params, registered_variables, state)."""
    wall = BoundarySettings1D(REFLECTIVE_BOUNDARY, REFLECTIVE_BOUNDARY)
    cfg = SimulationConfig(self_gravity=True, self_gravity_version=version, dimensionality=3, box_size=4.0,
                           num_cells=n, split=SPLIT, limiter=MINMOD, time_integrator=MUSCL, riemann_solver=HLLC,
                           boundary_settings=BoundarySettings(wall, wall, wall))
    rv = get_registered_variables(cfg)
    r = get_helper_data(cfg).r
    rho = np.where(r <= 1.0, 1.0 / (2 * np.pi * r), 1e-4)
    p = (5 / 3 - 1) * rho * 0.05
    z = np.zeros_like(rho)
    s = construct_primitive_state(cfg, rv, density=rho.astype(dtype), velocity_x=z, velocity_y=z, velocity_z=z,
                                  gas_pressure=p)
    cfg = finalize_config(cfg, s.shape)
    prm = SimulationParams(t_end=t_end, C_cfl=0.4, gamma=5 / 3, gravitational_constant=1.0)
    return cfg, prm, rv, s
