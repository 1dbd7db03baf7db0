"""Row layout of the state array (the variable registry).

Mirrors astronomix/variable_registry/registered_variables.py:43-238 field for
field, because the row indices are the data contract between a user's
initial-condition code and the CUDA kernels:

* 1D:       rho, u, p                                  (3 rows)
* 2D:       rho, vx, vy, p [, Bx, By, Bz at 4,5,6]      (4 / 7 rows)
* 3D:       rho, vx, vy, vz, p [, Bx, By, Bz at 5,6,7]  (5 / 8 rows)
* FD MHD:   + face fields bx, by, bz at rows 8, 9, 10   (11 rows)

The kernels index rows through the same numbers (``amx_layout`` in
include/amx.h is filled from this object).
"""

from typing import NamedTuple, Union

from .option_classes import FINITE_DIFFERENCE, XAXIS, YAXIS, ZAXIS, SimulationConfig


class StaticIntVector(NamedTuple):
    x: int
    y: int
    z: int


class AxisInfo(NamedTuple):
    axis_in_array: int
    velocity_index: int
    magnetic_index: int


class RegisteredVariables(NamedTuple):
    axes_info: tuple = ()
    num_vars: int = 3
    density_index: int = 0
    velocity_index: Union[int, StaticIntVector] = 1
    momentum_index: Union[int, StaticIntVector] = 1
    magnetic_index: Union[int, StaticIntVector] = -1
    interface_magnetic_field_index: Union[int, StaticIntVector] = -1
    pressure_index: int = 2
    energy_index: int = 2
    wind_density_index: int = -1
    wind_density_active: bool = False
    cosmic_ray_n_index: int = -1
    cosmic_ray_n_active: bool = False


def get_registered_variables(config: SimulationConfig) -> RegisteredVariables:
    """Registry for ``config`` (registered_variables.py:116-238)."""
    rv = RegisteredVariables()

    if config.dimensionality == 2:
        rv = rv._replace(num_vars=rv.num_vars + 1)
        rv = rv._replace(velocity_index=StaticIntVector(1, 2, -1))
        if config.mhd:
            rv = rv._replace(pressure_index=3)
            rv = rv._replace(magnetic_index=StaticIntVector(4, 5, 6))
            rv = rv._replace(num_vars=rv.num_vars + 3)
        else:
            rv = rv._replace(pressure_index=rv.num_vars - 1)

    if config.dimensionality == 3:
        rv = rv._replace(num_vars=rv.num_vars + 2)
        rv = rv._replace(velocity_index=StaticIntVector(1, 2, 3))
        rv = rv._replace(pressure_index=rv.num_vars - 1)
        if config.mhd:
            rv = rv._replace(magnetic_index=StaticIntVector(5, 6, 7))
            rv = rv._replace(num_vars=rv.num_vars + 3)

    if config.mhd and config.solver_mode == FINITE_DIFFERENCE:
        rv = rv._replace(
            interface_magnetic_field_index=StaticIntVector(
                rv.num_vars, rv.num_vars + 1, rv.num_vars + 2
            )
        )
        rv = rv._replace(num_vars=rv.num_vars + 3)

    if config.wind_config.trace_wind_density:
        rv = rv._replace(wind_density_index=rv.num_vars, num_vars=rv.num_vars + 1,
                         wind_density_active=True)

    if config.cosmic_ray_config.cosmic_rays:
        rv = rv._replace(cosmic_ray_n_index=rv.num_vars, num_vars=rv.num_vars + 1,
                         cosmic_ray_n_active=True)

    if config.dimensionality == 3 and config.mhd:
        rv = rv._replace(
            axes_info=(
                AxisInfo(XAXIS, rv.velocity_index.x, rv.magnetic_index.x),
                AxisInfo(YAXIS, rv.velocity_index.y, rv.magnetic_index.y),
                AxisInfo(ZAXIS, rv.velocity_index.z, rv.magnetic_index.z),
            )
        )

    rv = rv._replace(momentum_index=rv.velocity_index)
    rv = rv._replace(energy_index=rv.pressure_index)
    return rv
