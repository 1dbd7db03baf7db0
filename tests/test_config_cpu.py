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


def test_physics_switches_reach_the_c_structs():
    """self-gravity, the wind and the forcing: config and params fields land in
    amx_config / amx_params, and the limiter rewrite of finalize_config."""
    from astronomix_gb300 import SimulationParams, VAN_ALBADA, MINMOD, RIEMANN_SPLIT, _native
    from astronomix_gb300.option_classes import (WindConfig, WindParams, TurbulentForcingConfig,
                                                 TurbulentForcingParams)

    P = PERIODIC_BOUNDARY
    per = BoundarySettings(*[BoundarySettings1D(P, P)] * 3)
    cfg = finalize_config(SimulationConfig(dimensionality=3, self_gravity=True, self_gravity_version=RIEMANN_SPLIT,
                                           limiter=VAN_ALBADA, boundary_settings=per), (5, 8, 8, 8))
    assert cfg.limiter == MINMOD  # simulation_config.py:384-389
    c = make_amx_config(cfg, get_registered_variables(cfg), (5, 8, 8, 8), np.float32)
    assert c.self_gravity == 1 and c.self_gravity_version == RIEMANN_SPLIT
    cfg = SimulationConfig(dimensionality=3, mhd=True, solver_mode=FINITE_DIFFERENCE, boundary_settings=per,
                           wind_config=WindConfig(stellar_wind=True, num_injection_cells=6),
                           turbulent_forcing_config=TurbulentForcingConfig(turbulent_forcing=True))
    cfg = finalize_config(cfg, (11, 8, 8, 8))
    c = make_amx_config(cfg, get_registered_variables(cfg), (11, 8, 8, 8), np.float64)
    assert (c.stellar_wind, c.num_injection_cells, c.turbulent_forcing) == (1, 6, 1)
    prm = SimulationParams(gravitational_constant=3.0,
                           wind_params=WindParams(wind_mass_loss_rate=2.0, wind_final_velocity=5.0),
                           turbulent_forcing_params=TurbulentForcingParams(energy_injection_rate=0.7))
    p = _native.make_params(prm)
    assert (p.gravitational_constant, p.wind_mass_loss_rate, p.wind_final_velocity, p.energy_injection_rate,
            p.forcing_seed) == (3.0, 2.0, 5.0, 0.7, 42)


def test_unsupported_physics_raise_before_any_gpu_work():
    from astronomix_gb300.time_integration import _check_supported
    from astronomix_gb300.option_classes import WindConfig, TurbulentForcingConfig

    P = PERIODIC_BOUNDARY
    per = BoundarySettings(*[BoundarySettings1D(P, P)] * 3)
    with pytest.raises(NotImplementedError):  # the FV wind is the physics-module injection
        _check_supported(SimulationConfig(dimensionality=3, wind_config=WindConfig(stellar_wind=True)))
    with pytest.raises(NotImplementedError):  # self-gravity is an FV feature
        _check_supported(SimulationConfig(dimensionality=3, mhd=True, solver_mode=FINITE_DIFFERENCE,
                                          self_gravity=True, boundary_settings=per))
    with pytest.raises(ValueError):  # the forcing field has the unpadded grid's shape
        _check_supported(SimulationConfig(dimensionality=3,
                                          turbulent_forcing_config=TurbulentForcingConfig(turbulent_forcing=True)))
    _check_supported(SimulationConfig(dimensionality=3, boundary_handling=PERIODIC_ROLL, boundary_settings=per,
                                      turbulent_forcing_config=TurbulentForcingConfig(turbulent_forcing=True)))


def test_initialize_interface_fields_matches_oracle():
    """The host-side face-field initialisation (_constrained_transport.py:202-213,
    4th-order centre-to-face interpolation) equals the oracle's bit for bit."""
    import numpy as np
    from astronomix_gb300 import initialize_interface_fields
    from oracle import fd as ofd

    rng = np.random.default_rng(11)
    B = [rng.standard_normal((12, 10, 8)) for _ in range(3)]
    got = initialize_interface_fields(*B)
    ref = ofd.initialize_interface_fields(*B)
    for g, r in zip(got, ref):
        assert g.shape == r.shape
        assert np.array_equal(g, r)
