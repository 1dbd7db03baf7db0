"""Set-up helpers of the public API (host side, not on the accelerated path).

* get_helper_data            -- astronomix/data_classes/simulation_helper_data.py:49-160
* construct_primitive_state  -- astronomix/initial_condition_generation/construct_primitive_state.py:18-116
* initialize_interface_fields -- astronomix/_finite_difference/_magnetic_update/_constrained_transport.py:202-213

These run once per simulation on the host (NumPy), like the reference's
set-up code, and produce arrays in the reference's layout.
"""

from typing import NamedTuple, Any

import numpy as np

from .option_classes import CARTESIAN, FINITE_DIFFERENCE, SimulationConfig
from .variable_registry import RegisteredVariables


class HelperData(NamedTuple):
    geometric_centers: Any = None
    volumetric_centers: Any = None
    r: Any = None
    r_hat_alpha: Any = None
    cell_volumes: Any = None
    inner_cell_boundaries: Any = None
    outer_cell_boundaries: Any = None


def get_helper_data(config: SimulationConfig, sharding=None, padded: bool = False,
                    production: bool = False) -> HelperData:
    """Cell centres, radii and volumes (simulation_helper_data.py:49-160).

    As in the reference, the 2D/3D centres come from ``meshgrid`` with its
    default 'xy' indexing, so ``geometric_centers[..., 0]`` varies along the
    second array axis.
    """
    if config.geometry != CARTESIAN:
        raise NotImplementedError("only Cartesian geometry is part of the accelerated path")
    ngc = config.num_ghost_cells if padded else 0
    dx = config.box_size / config.num_cells
    if production:
        return HelperData()
    n = config.num_cells + 2 * ngc
    if config.dimensionality > 1:
        x = np.linspace(dx / 2 - ngc * dx, config.box_size + dx / 2 + ngc * dx, n, endpoint=False)
        if config.dimensionality == 3:
            gc = np.array(np.meshgrid(x, x, x))
        else:
            gc = np.array(np.meshgrid(x, x))
        gc = np.moveaxis(gc, 0, -1)
        box_center = np.zeros(config.dimensionality) + config.box_size / 2
        r = np.linalg.norm(gc - box_center, axis=-1)
        return HelperData(geometric_centers=gc, volumetric_centers=gc, r=r)
    r = np.linspace(dx / 2 - ngc * dx, config.box_size - dx / 2 + ngc * dx, n)
    return HelperData(
        geometric_centers=r,
        volumetric_centers=r,
        r_hat_alpha=dx * np.ones_like(r),
        cell_volumes=dx * np.ones_like(r),
        inner_cell_boundaries=r - dx / 2,
        outer_cell_boundaries=r + dx / 2,
    )


def construct_primitive_state(config: SimulationConfig, registered_variables: RegisteredVariables,
                              density, velocity_x=None, velocity_y=None, velocity_z=None,
                              magnetic_field_x=None, magnetic_field_y=None, magnetic_field_z=None,
                              interface_magnetic_field_x=None, interface_magnetic_field_y=None,
                              interface_magnetic_field_z=None, gas_pressure=None,
                              cosmic_ray_pressure=None, sharding=None):
    """Stack the fields into the state array (construct_primitive_state.py:18-116).

    The dtype of the result is the dtype of ``density`` (float32 or float64);
    it selects the precision of the CUDA kernels.
    """
    rv = registered_variables
    density = np.asarray(density)
    dtype = density.dtype if density.dtype in (np.float32, np.float64) else np.float32
    state = np.zeros((rv.num_vars, *density.shape), dtype=dtype)
    state[rv.density_index] = density
    d = config.dimensionality
    if d == 1:
        state[rv.velocity_index] = velocity_x
    elif d == 2:
        state[rv.velocity_index.x] = velocity_x
        state[rv.velocity_index.y] = velocity_y
    elif d == 3:
        state[rv.velocity_index.x] = velocity_x
        state[rv.velocity_index.y] = velocity_y
        state[rv.velocity_index.z] = velocity_z
    if config.mhd and d >= 2:
        if magnetic_field_x is not None:
            state[rv.magnetic_index.x] = magnetic_field_x
        if magnetic_field_y is not None:
            state[rv.magnetic_index.y] = magnetic_field_y
        if magnetic_field_z is not None:
            state[rv.magnetic_index.z] = magnetic_field_z
        if config.solver_mode == FINITE_DIFFERENCE:
            if interface_magnetic_field_x is not None:
                state[rv.interface_magnetic_field_index.x] = interface_magnetic_field_x
            if interface_magnetic_field_y is not None:
                state[rv.interface_magnetic_field_index.y] = interface_magnetic_field_y
            if interface_magnetic_field_z is not None:
                state[rv.interface_magnetic_field_index.z] = interface_magnetic_field_z
    state[rv.pressure_index] = gas_pressure
    if rv.cosmic_ray_n_active:
        raise NotImplementedError("cosmic rays are not part of the accelerated path")
    return state


def _c2f(a, axis):
    # (-f[i-1] + 9 f[i] + 9 f[i+1] - f[i+2]) / 16 with periodic wrap
    return (-np.roll(a, 1, axis) + 9 * a + 9 * np.roll(a, -1, axis) - np.roll(a, -2, axis)) / 16.0


def initialize_interface_fields(magnetic_field_x, magnetic_field_y, magnetic_field_z):
    """Face magnetic fields from cell-centred ones, 4th order (_constrained_transport.py:202-213)."""
    return (_c2f(np.asarray(magnetic_field_x), 0), _c2f(np.asarray(magnetic_field_y), 1),
            _c2f(np.asarray(magnetic_field_z), 2))
