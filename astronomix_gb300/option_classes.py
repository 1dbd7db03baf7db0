"""Static configuration and traced parameters of a simulation.

Mirrors the contract of astronomix's option classes so that existing driver
scripts build the same objects with the same field names, defaults and
integer constants:

* constants            -- astronomix/option_classes/simulation_config.py:20-93
* SnapshotSettings     -- astronomix/option_classes/simulation_config.py:117-146
* BoundarySettings*    -- astronomix/option_classes/simulation_config.py:149-157
* SimulationConfig     -- astronomix/option_classes/simulation_config.py:160-342
* finalize_config      -- astronomix/option_classes/simulation_config.py:345-470
* SimulationParams     -- astronomix/option_classes/simulation_params.py:11-66

The config selects which CUDA kernel instantiation runs (solver, limiter,
dimensionality, precision); the params are passed to the kernels as plain
numbers.  Self-gravity (finite volume), turbulent forcing (3D) and the
stellar-wind source of the finite-difference scheme run on the GPU with the
step.  The other physics modules (cooling, cosmic rays, learned forces, the
finite-volume wind injection) are outside the accelerated MHD step: their
option classes exist so that configs built for astronomix still construct,
and switching one on raises ``NotImplementedError`` in ``time_integration``.
"""

from typing import NamedTuple, Union, Any

# ===================== constant definition =====================

# solver modes
FINITE_VOLUME = 0
FINITE_DIFFERENCE = 1

# differentiation modes
FORWARDS = 0
BACKWARDS = 1

# limiter types
MINMOD = 0
OSHER = 1
DOUBLE_MINMOD = 2
SUPERBEE = 3
VAN_ALBADA = 4
VAN_ALBADA_PP = 5

# splitting modes
UNSPLIT = 0
SPLIT = 1

# Riemann solvers
HLL = 0
HLLC = 1
HLLC_LM = 2
LAX_FRIEDRICHS = 3
HYBRID_HLLC = 4
AM_HLLC = 5

# time integrators
RK2_SSP = 0
MUSCL = 1
RK4_SSP = 2

# boundary conditions
OPEN_BOUNDARY = 0
REFLECTIVE_BOUNDARY = 1
PERIODIC_BOUNDARY = 2
MHD_JET_BOUNDARY = 3

GAS_STATE = 0
VELOCITY_ONLY = 1
MAGNETIC_FIELD_ONLY = 2

# geometry types
CARTESIAN = 0
CYLINDRICAL = 1
SPHERICAL = 2

# axes
VARAXIS = 0
XAXIS = 1
YAXIS = 2
ZAXIS = 3

# boundary handling modes
GHOST_CELLS = 0
PERIODIC_ROLL = 1

# self-gravity versions
SIMPLE_SOURCE_TERM = 0
DONOR_ACCOUNTING = 1
RIEMANN_SPLIT = 2
RIEMANN_SPLIT_UNSTABLE = 3
HALF_SPLIT = 4

# magnetic part integrators for split MHD
IMPLICIT_MIDPOINT = 0
IMPLICIT_EULER = 1

# numerical precision (selects the fixed-point tolerance of the FV magnetic
# sub-step, exactly as in the reference; the arithmetic type is chosen by the
# dtype of the state array handed to time_integration)
SINGLE_PRECISION = 0
DOUBLE_PRECISION = 1

STATE_TYPE = Any


# ============ physics-module option placeholders (off-path) ============

class TurbulentForcingConfig(NamedTuple):
    turbulent_forcing: bool = False


class TurbulentForcingParams(NamedTuple):
    energy_injection_rate: float = 2.0


class WindConfig(NamedTuple):
    stellar_wind: bool = False
    num_injection_cells: int = 10
    wind_injection_scheme: int = 1
    trace_wind_density: bool = False


class WindParams(NamedTuple):
    wind_mass_loss_rate: float = 0.0
    wind_final_velocity: float = 0.0
    pressure_floor: float = 100000.0


class CosmicRayConfig(NamedTuple):
    cosmic_rays: bool = False
    diffusive_shock_acceleration: bool = False


class CosmicRayParams(NamedTuple):
    diffusive_shock_acceleration_start_time: float = 0.0
    diffusive_shock_acceleration_efficiency: float = 0.1


class CoolingConfig(NamedTuple):
    cooling: bool = False
    cooling_method: int = 2
    cooling_curve_config: Any = None


class CoolingParams(NamedTuple):
    hydrogen_mass_fraction: float = 0.76
    metal_mass_fraction: float = 0.02
    floor_temperature: float = 1e4
    cooling_curve_params: Any = None


class NeuralNetForceConfig(NamedTuple):
    neural_net_force: bool = False
    network_static: Any = None


class NeuralNetForceParams(NamedTuple):
    network_params: Any = None


class CNNMHDconfig(NamedTuple):
    cnn_mhd_corrector: bool = False
    network_static: Any = None


class CNNMHDParams(NamedTuple):
    network_params: Any = None


# ===================== snapshot / boundary settings =====================

class SnapshotSettings(NamedTuple):
    """Which diagnostics are recorded at snapshot times."""

    return_states: bool = True
    return_final_state: bool = False
    return_total_mass: bool = False
    return_total_energy: bool = False
    return_internal_energy: bool = False
    return_kinetic_energy: bool = False
    return_gravitational_energy: bool = False
    return_radial_momentum: bool = False
    return_magnetic_divergence: bool = False


class BoundarySettings1D(NamedTuple):
    left_boundary: int = OPEN_BOUNDARY
    right_boundary: int = OPEN_BOUNDARY


class BoundarySettings(NamedTuple):
    x: BoundarySettings1D = BoundarySettings1D()
    y: BoundarySettings1D = BoundarySettings1D()
    z: BoundarySettings1D = BoundarySettings1D()


# ===================== the configuration =====================

class SimulationConfig(NamedTuple):
    """Static simulation configuration (a change selects other kernels)."""

    solver_mode: int = FINITE_VOLUME
    numerical_precision: int = SINGLE_PRECISION
    runtime_debugging: bool = False
    donate_state: bool = False
    memory_analysis: bool = False
    print_elapsed_time: bool = False
    progress_bar: bool = False
    dimensionality: int = 1
    state_struct: bool = False
    geometry: int = CARTESIAN
    mhd: bool = False
    fv_magnetic_integrator: int = IMPLICIT_MIDPOINT
    enforce_positivity: bool = True
    self_gravity: bool = False
    self_gravity_version: int = DONOR_ACCOUNTING
    box_size: float = 1.0
    num_cells: int = 400
    reconstruction_order: int = 1
    limiter: int = MINMOD
    riemann_solver: int = HLL
    split: int = UNSPLIT
    time_integrator: int = RK2_SSP
    # evaluated at class-definition time in the reference as well
    # (reconstruction_order + 1 = 2, box_size / num_cells = 1 / 400)
    num_ghost_cells: int = 2
    grid_spacing: float = 1.0 / 400
    boundary_handling: int = GHOST_CELLS
    boundary_settings: Union[None, BoundarySettings1D, BoundarySettings] = None
    fixed_timestep: bool = False
    exact_end_time: bool = True
    source_term_aware_timestep: bool = False
    num_timesteps: int = 1000
    use_max_adaptive_timestep: bool = True
    differentiation_mode: int = FORWARDS
    num_checkpoints: int = 100
    return_snapshots: bool = False
    snapshot_settings: SnapshotSettings = SnapshotSettings()
    activate_snapshot_callback: bool = False
    use_specific_snapshot_timepoints: bool = False
    num_snapshots: int = 10
    first_order_fallback: bool = False
    turbulent_forcing_config: TurbulentForcingConfig = TurbulentForcingConfig()
    wind_config: WindConfig = WindConfig()
    cosmic_ray_config: CosmicRayConfig = CosmicRayConfig()
    cooling_config: CoolingConfig = CoolingConfig()
    neural_net_force_config: NeuralNetForceConfig = NeuralNetForceConfig()
    cnn_mhd_corrector_config: CNNMHDconfig = CNNMHDconfig()


class SimulationParams(NamedTuple):
    """Parameters that change no kernel (passed as kernel arguments)."""

    C_cfl: float = 0.4
    gravitational_constant: float = 1.0
    gamma: float = 5 / 3
    minimum_density: float = 1e-14
    minimum_pressure: float = 1e-14
    dt_max: float = 0.001
    t_end: float = 0.2
    snapshot_timepoints: Any = (0.0,)
    turbulent_forcing_params: TurbulentForcingParams = TurbulentForcingParams()
    wind_params: WindParams = WindParams()
    cosmic_ray_params: CosmicRayParams = CosmicRayParams()
    cooling_params: CoolingParams = CoolingParams()
    neural_net_force_params: NeuralNetForceParams = NeuralNetForceParams()
    cnn_mhd_corrector_params: CNNMHDParams = CNNMHDParams()


_PERIODIC_3D = BoundarySettings(
    BoundarySettings1D(PERIODIC_BOUNDARY, PERIODIC_BOUNDARY),
    BoundarySettings1D(PERIODIC_BOUNDARY, PERIODIC_BOUNDARY),
    BoundarySettings1D(PERIODIC_BOUNDARY, PERIODIC_BOUNDARY),
)


def finalize_config(config: SimulationConfig, state_shape) -> SimulationConfig:
    """Validate the config and apply the reference's automatic rewrites.

    Follows astronomix/option_classes/simulation_config.py:345-470: sets
    ``num_cells`` from the state shape, requires square/cubic grids, resets
    ``grid_spacing``, forces SSPRK(5,4) and periodic roll for the finite
    difference scheme and fills in default boundary settings.
    """
    num_cells = state_shape[-1]
    config = config._replace(num_cells=num_cells)

    if config.dimensionality == 2:
        nx, ny = state_shape[-2:]
        if nx != ny:
            raise ValueError("The number of cells in x and y must be equal.")
    elif config.dimensionality == 3:
        nx, ny, nz = state_shape[-3:]
        if nx != ny or nx != nz:
            raise ValueError("The number of cells in x, y and z must be equal.")

    config = config._replace(grid_spacing=config.box_size / config.num_cells)

    if config.geometry == SPHERICAL:
        print("For spherical geometry, only HLL is currently supported. Also, only the unsplit mode has been tested.")
        if config.riemann_solver != HLL:
            print("Setting HLL Riemann solver for spherical geometry.")
            config = config._replace(riemann_solver=HLL)
        if config.split != SPLIT:
            print("Setting unsplit mode for spherical geometry")
            config = config._replace(split=SPLIT)
        if config.limiter in (VAN_ALBADA, VAN_ALBADA_PP):
            print("Setting minmod limiter for spherical geometry")
            config = config._replace(limiter=MINMOD)
        if config.time_integrator != MUSCL:
            print("Setting MUSCL time integrator for spherical geometry")
            config = config._replace(time_integrator=MUSCL)

    if config.self_gravity and config.limiter != MINMOD:
        print("Setting DOUBLE_MINMOD limiter for self-gravity.")
        config = config._replace(limiter=MINMOD)

    if config.solver_mode == FINITE_DIFFERENCE:
        if not config.mhd:
            raise ValueError(
                "Finite difference solver mode is currently only supported for MHD simulations."
            )
        if config.dimensionality != 3:
            raise ValueError(
                "Finite difference solver mode is currently only supported for 3D simulations."
            )
        if config.boundary_settings != _PERIODIC_3D:
            raise ValueError(
                "Finite difference solver mode currently only supports periodic boundaries."
            )
        if config.time_integrator != RK4_SSP:
            print("Setting time integrator to RK4_SSP for finite difference solver mode.")
            config = config._replace(time_integrator=RK4_SSP)
        if config.boundary_handling != PERIODIC_ROLL:
            print("Setting boundary handling to PERIODIC_ROLL for finite difference solver mode.")
            config = config._replace(boundary_handling=PERIODIC_ROLL)

    if config.boundary_settings is None:
        if config.geometry == CARTESIAN:
            print("Automatically setting open boundaries for Cartesian geometry.")
            if config.dimensionality == 1:
                config = config._replace(
                    boundary_settings=BoundarySettings1D(OPEN_BOUNDARY, OPEN_BOUNDARY)
                )
            else:
                config = config._replace(boundary_settings=BoundarySettings())
        elif config.geometry == SPHERICAL and config.dimensionality == 1:
            config = config._replace(
                boundary_settings=BoundarySettings1D(REFLECTIVE_BOUNDARY, OPEN_BOUNDARY)
            )

    if config.wind_config.stellar_wind:
        print("For stellar wind simulations, we need source term aware timesteps, turning on.")
        config = config._replace(source_term_aware_timestep=True)

    return config
