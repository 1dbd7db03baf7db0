"""Host logic without a GPU: the config / registry mirror and the C-struct translation."""
import numpy as np
import pytest

from astronomix_gb300 import (
    SimulationConfig, get_registered_variables, finalize_config, BoundarySettings, BoundarySettings1D,
    FINITE_DIFFERENCE, PERIODIC_BOUNDARY, OPEN_BOUNDARY, HLLC, RK4_SSP, PERIODIC_ROLL,
)
from astronomix_gb300.time_integration import make_amx_config


def test_registry_layouts_match_reference():
    # registered_variables.py:116-238
    rv = get_registered_variables(SimulationConfig(dimensionality=1))
    assert (rv.num_vars, rv.density_index, rv.velocity_index, rv.pressure_index) == (3, 0, 1, 2)
    rv = get_registered_variables(SimulationConfig(dimensionality=2, mhd=True))
    assert rv.num_vars == 7 and rv.pressure_index == 3 and tuple(rv.magnetic_index) == (4, 5, 6)
    rv = get_registered_variables(SimulationConfig(dimensionality=3, mhd=True))
    assert rv.num_vars == 8 and rv.pressure_index == 4 and tuple(rv.magnetic_index) == (5, 6, 7)
    rv = get_registered_variables(SimulationConfig(dimensionality=3, mhd=True, solver_mode=FINITE_DIFFERENCE))
    assert rv.num_vars == 11 and tuple(rv.interface_magnetic_field_index) == (8, 9, 10)
    assert rv.momentum_index == rv.velocity_index and rv.energy_index == rv.pressure_index


def test_finalize_config_rewrites_and_errors():
    P = PERIODIC_BOUNDARY
    per = BoundarySettings(*[BoundarySettings1D(P, P)] * 3)
    cfg = finalize_config(SimulationConfig(dimensionality=3, mhd=True, solver_mode=FINITE_DIFFERENCE,
                                           boundary_settings=per), (11, 16, 16, 16))
    assert cfg.time_integrator == RK4_SSP and cfg.boundary_handling == PERIODIC_ROLL
    assert cfg.num_cells == 16 and cfg.grid_spacing == 1.0 / 16
    with pytest.raises(ValueError):
        finalize_config(SimulationConfig(dimensionality=2), (4, 16, 8))
    with pytest.raises(ValueError):
        finalize_config(SimulationConfig(dimensionality=2, solver_mode=FINITE_DIFFERENCE, mhd=True), (7, 8, 8))
    with pytest.raises(ValueError):
        finalize_config(SimulationConfig(dimensionality=3, solver_mode=FINITE_DIFFERENCE, mhd=True), (11, 8, 8, 8))
    cfg = finalize_config(SimulationConfig(dimensionality=1), (3, 10))
    assert cfg.boundary_settings == BoundarySettings1D(OPEN_BOUNDARY, OPEN_BOUNDARY)


def test_make_amx_config_translation():
    P = PERIODIC_BOUNDARY
    cfg = finalize_config(SimulationConfig(dimensionality=2, mhd=True, riemann_solver=HLLC, box_size=2.0,
                                           boundary_settings=BoundarySettings(BoundarySettings1D(P, P),
                                                                              BoundarySettings1D(OPEN_BOUNDARY,
                                                                                                 OPEN_BOUNDARY))),
                          (7, 32, 32))
    rv = get_registered_variables(cfg)
    c = make_amx_config(cfg, rv, (7, 32, 32), np.float32)
    assert (c.dimensionality, c.num_cells, c.num_vars, c.mhd, c.riemann_solver) == (2, 32, 7, 1, HLLC)
    assert list(c.bc_lo)[:2] == [P, OPEN_BOUNDARY] and list(c.bc_hi)[:2] == [P, OPEN_BOUNDARY]
    assert c.dtype == 0 and c.grid_spacing == pytest.approx(2.0 / 32)
    assert make_amx_config(cfg, rv, (7, 32, 32), np.float64).dtype == 1
