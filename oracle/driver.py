"""Oracle: restatement of the reference's time driver (test infrastructure).

Follows astronomix/time_stepping/time_integration.py:239-845 for the
configurations on the accelerated path: padding with 2 edge cells, the gas
ghost-cell fill, the adaptive (or fixed) time step with exact end time, the
finite-volume / finite-difference evolve, and the unpad.  Snapshot
diagnostics follow :404-537 (mass, energy, kinetic/internal energy, max |div
B|).

``time_mode="reference"`` keeps the time accumulator and dt in the state
dtype, like the reference; ``"float64"`` keeps them in float64, which is what
the CUDA driver does (FP32 fields, FP64 time and dt reduction).
"""

from types import SimpleNamespace

import numpy as np

from astronomix_gb300.option_classes import (
    GHOST_CELLS, FINITE_VOLUME, FINITE_DIFFERENCE,
)
from ._xp import xp
from . import fv as _fv
from . import fd as _fd


def _dtype_scalar(v, like, time_mode):
    if time_mode == "float64":
        return xp.to_float(v)  # detached, like the reference's stop_gradient(dt)
    return xp.scalar(v, like)


def cfl_dt(P, config, params, rv, time_mode="reference"):
    """One adaptive time step (time_integration.py:629-666)."""
    if config.solver_mode == FINITE_VOLUME:
        dt = _fv.cfl_time_step(P, config.grid_spacing, params.dt_max, params.gamma, config, rv, params.C_cfl)
    else:
        dt = _fd.cfl_time_step_fd(P, config.grid_spacing, params.dt_max, params.gamma, params.C_cfl,
                                  params.minimum_density, params.minimum_pressure)
    return _dtype_scalar(dt, P, time_mode)


def evolve(P, dt, config, params, rv, stats=None):
    gamma = xp.scalar(params.gamma, P)
    if config.solver_mode == FINITE_VOLUME:
        dt_ = xp.scalar(dt, P)
        return _fv.evolve_state_fv(P, dt_, gamma, config, rv, stats=stats, C_cfl=xp.scalar(params.C_cfl, P),
                                   G=params.gravitational_constant)
    wind = None
    if config.wind_config.stellar_wind:
        from .forcing import cell_radius
        wp = params.wind_params
        wind = (wp.wind_mass_loss_rate, wp.wind_final_velocity,
                cell_radius(config.num_cells, config.grid_spacing, config.box_size),
                config.wind_config.num_injection_cells)
    return _fd.evolve_state_fd(P, dt, gamma, config.grid_spacing, params.minimum_density,
                               params.minimum_pressure, config.enforce_positivity, wind)


def snapshot_quantities(P_unpadded, config, params, rv):
    """Diagnostics of time_integration.py:404-537 (Cartesian, no gravity)."""
    d = config.dimensionality
    dV = config.grid_spacing ** d
    gamma = params.gamma
    rho = P_unpadded[rv.density_index]
    p = P_unpadded[rv.pressure_index]
    if config.solver_mode == FINITE_DIFFERENCE:
        u = xp.sqrt(P_unpadded[1] ** 2 + P_unpadded[2] ** 2 + P_unpadded[3] ** 2 + 1e-20)
    else:
        u = _fv.get_absolute_velocity(P_unpadded, d, rv)
    out = SimpleNamespace()
    if d == 1:
        dv = config.grid_spacing
        out.total_mass = float(xp.to_float((rho * dv).sum()))
    else:
        out.total_mass = float(xp.to_float(rho.sum())) * config.box_size ** d
    out.total_energy = float(xp.to_float(_fv.total_energy_from_primitives(rho, u, p, gamma).sum())) * (
        config.grid_spacing if d == 1 else dV)
    out.internal_energy = float(xp.to_float((p / (gamma - 1)).sum())) * (config.grid_spacing if d == 1 else dV)
    out.kinetic_energy = float(xp.to_float((0.5 * rho * u ** 2).sum())) * (config.grid_spacing if d == 1 else dV)
    if config.mhd:
        if config.solver_mode == FINITE_DIFFERENCE:
            div = _fd.interface_field_divergence(P_unpadded[8], P_unpadded[9], P_unpadded[10], config.grid_spacing)
        else:
            mi = rv.magnetic_index
            div = _fv.divergence(P_unpadded[mi.x:mi.z + 1], config.grid_spacing, d)
        out.magnetic_divergence = float(xp.to_float(xp.amax(xp.abs(div))))
    return out


def time_integration(state, config, params, rv, time_mode="reference", max_steps=None,
                     record=None):
    """Integrate to ``params.t_end`` (or ``max_steps`` steps).

    ``record`` (a dict, optional) receives ``dts`` (list of floats),
    ``magnetic_iterations`` (list of ints, FV MHD) and ``steps``.
    """
    d = config.dimensionality
    ghost = config.boundary_handling == GHOST_CELLS
    P = state
    if ghost:
        P = _fv.pad(P, d)
        if config.mhd:
            P = xp.copy(P)
            P[:-3] = _fv.boundary_handler(P[:-3], config)
        else:
            P = _fv.boundary_handler(P, config)

    t = _dtype_scalar(0.0, P, time_mode)
    t_end = params.t_end
    steps = 0
    dts, its = [], []
    while True:
        if max_steps is not None and steps >= max_steps:
            break
        if config.fixed_timestep:
            if steps >= config.num_timesteps:
                break
        elif not (t < t_end):
            break
        if config.fixed_timestep:
            dt = _dtype_scalar(params.t_end / config.num_timesteps, P, time_mode)
        else:
            dt = cfl_dt(P, config, params, rv, time_mode)
            if config.exact_end_time:
                dt = min(dt, _dtype_scalar(t_end, P, time_mode) - t) if time_mode == "float64" else \
                    xp.minimum(dt, xp.scalar(t_end, P) - t)
        if config.turbulent_forcing_config.turbulent_forcing:
            # time_integration.py:700-711 (Philox noise, see oracle/forcing.py)
            if ghost:
                raise ValueError("turbulent forcing needs the unpadded state (periodic roll)")
            from .forcing import apply_forcing
            P = apply_forcing(P, dt, steps, config, params, rv)
        P = evolve(P, dt, config, params, rv, stats=its)
        t = t + dt
        dts.append(float(dt))
        steps += 1
    if record is not None:
        record["dts"] = dts
        record["magnetic_iterations"] = its
        record["steps"] = steps
        record["t"] = float(t)
    if ghost:
        P = _fv.unpad(P, d)
    return P


def as_array(x, dtype=np.float64):
    return np.asarray(x, dtype=dtype)
