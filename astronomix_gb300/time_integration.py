"""The drop-in time driver: ``time_integration(state, config, params, rv)``.

Same signature and return types as astronomix's time_integration
(astronomix/time_stepping/time_integration.py:61-236).  The state may be a
NumPy array or a torch tensor (CPU or CUDA), float32 or float64; the result
comes back in the same form.  The whole loop runs on the GPU through the C
ABI (include/amx.h): the host only launches and, when snapshots are
requested, pauses at the snapshot times.
"""

from typing import NamedTuple, Any
import math

import numpy as np

from . import _native
from .option_classes import (
    FINITE_VOLUME, FINITE_DIFFERENCE, GHOST_CELLS, PERIODIC_ROLL, PERIODIC_BOUNDARY, OPEN_BOUNDARY,
    UNSPLIT, SPLIT, RK2_SSP, MUSCL, CARTESIAN, SimulationConfig, SimulationParams, BoundarySettings1D,
)
from .variable_registry import RegisteredVariables


class SnapshotData(NamedTuple):
    """Return format when snapshots are requested (data_classes/simulation_snapshot_data.py:5-45)."""

    time_points: Any = None
    states: Any = None
    final_state: Any = None
    total_mass: Any = None
    total_energy: Any = None
    internal_energy: Any = None
    kinetic_energy: Any = None
    gravitational_energy: Any = None
    radial_momentum: Any = None
    magnetic_divergence: Any = None
    runtime: float = 0.0
    num_iterations: int = 0
    current_checkpoint: int = 0


class StateStruct(NamedTuple):
    primitive_state: Any = None


def _check_supported(config: SimulationConfig):
    if config.geometry != CARTESIAN:
        raise NotImplementedError("only Cartesian geometry is part of the accelerated path")
    if config.self_gravity and config.solver_mode != FINITE_VOLUME:
        raise NotImplementedError("self-gravity is part of the finite-volume scheme only")
    if config.cooling_config.cooling or config.cosmic_ray_config.cosmic_rays or \
            config.neural_net_force_config.neural_net_force or config.cnn_mhd_corrector_config.cnn_mhd_corrector:
        raise NotImplementedError("physics modules are not part of the accelerated MHD step")
    if config.wind_config.stellar_wind and config.solver_mode != FINITE_DIFFERENCE:
        # the FD scheme's wind is a right-hand-side source (_ssprk.py:230-241); the FV
        # physics-module injection is not part of the accelerated path
        raise NotImplementedError("stellar wind is supported as the finite-difference source term")
    if config.turbulent_forcing_config.turbulent_forcing and (
            config.dimensionality != 3 or
            (config.solver_mode == FINITE_VOLUME and config.boundary_handling != PERIODIC_ROLL)):
        raise ValueError("turbulent forcing acts on the unpadded 3D state (periodic roll)")
    if config.solver_mode == FINITE_VOLUME:
        if config.split == UNSPLIT:
            if config.time_integrator != RK2_SSP:
                raise ValueError("Only the RK2 SSP time integrator is currently supported for the unsplit scheme.")
        elif config.split == SPLIT:
            if config.time_integrator != MUSCL and not config.first_order_fallback:
                raise ValueError("Time integrator %d not supported for split reconstruction. Only MUSCL is "
                                 "supported." % config.time_integrator)
        else:
            raise ValueError("unknown split mode %d" % config.split)


def _bc_codes(config: SimulationConfig):
    lo, hi = [PERIODIC_BOUNDARY] * 3, [PERIODIC_BOUNDARY] * 3
    bs = config.boundary_settings
    if bs is None:
        bs = BoundarySettings1D(OPEN_BOUNDARY, OPEN_BOUNDARY) if config.dimensionality == 1 else None
    if isinstance(bs, BoundarySettings1D):
        lo[0], hi[0] = bs.left_boundary, bs.right_boundary
    elif bs is not None:
        for k, b in enumerate((bs.x, bs.y, bs.z)):
            lo[k], hi[k] = b.left_boundary, b.right_boundary
    else:
        lo, hi = [OPEN_BOUNDARY] * 3, [OPEN_BOUNDARY] * 3
    return lo, hi


def make_amx_config(config: SimulationConfig, rv: RegisteredVariables, shape, dtype) -> _native.amx_config:
    """Translate a (finalised) SimulationConfig into the C struct."""
    c = _native.amx_config()
    c.solver_mode = int(config.solver_mode)
    c.dtype = _native.AMX_F64 if np.dtype(dtype) == np.float64 else _native.AMX_F32
    c.dimensionality = int(config.dimensionality)
    c.num_cells = int(shape[-1])
    c.num_vars = int(shape[0])
    c.mhd = int(bool(config.mhd))
    c.riemann_solver = int(config.riemann_solver)
    c.limiter = int(config.limiter)
    c.fv_magnetic_integrator = int(config.fv_magnetic_integrator)
    c.numerical_precision = int(config.numerical_precision)
    c.boundary_handling = int(config.boundary_handling)
    lo, hi = _bc_codes(config)
    for k in range(3):
        c.bc_lo[k] = int(lo[k])
        c.bc_hi[k] = int(hi[k])
    c.enforce_positivity = int(bool(config.enforce_positivity))
    # with specific snapshot time points, dt is clipped to the next time point
    # (time_integration.py:671-678): the driver passes that point as t_end
    c.exact_end_time = int(bool(config.exact_end_time) or
                           bool(config.use_specific_snapshot_timepoints and config.return_snapshots))
    c.fixed_timestep = int(bool(config.fixed_timestep))
    c.num_timesteps = int(config.num_timesteps)
    c.box_size = float(config.box_size)
    c.grid_spacing = float(config.grid_spacing)
    c.split = int(config.split)
    c.first_order_fallback = int(bool(config.first_order_fallback))
    c.use_max_adaptive_timestep = int(bool(config.use_max_adaptive_timestep))
    c.self_gravity = int(bool(config.self_gravity))
    c.self_gravity_version = int(config.self_gravity_version)
    c.stellar_wind = int(bool(config.wind_config.stellar_wind))
    c.num_injection_cells = int(config.wind_config.num_injection_cells)
    c.turbulent_forcing = int(bool(config.turbulent_forcing_config.turbulent_forcing))
    return c


_PLANS = {}


def get_plan(config, rv, shape, dtype, max_history=0):
    key = (config, rv, tuple(shape), np.dtype(dtype).str, int(max_history))
    plan = _PLANS.get(key)
    if plan is None:
        plan = _native.Plan(make_amx_config(config, rv, shape, dtype), max_history)
        _PLANS[key] = plan
    return plan


def _to_device(state):
    """-> (cuda tensor, restore function)."""
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("astronomix_gb300 runs on a CUDA GPU; no device is visible")
    if isinstance(state, torch.Tensor):
        was_cuda = state.is_cuda
        dev = state.detach().to("cuda").contiguous().clone()

        def restore(t):
            return t if was_cuda else t.cpu()

        return dev, restore
    arr = np.ascontiguousarray(state)
    if arr.dtype not in (np.float32, np.float64):
        arr = arr.astype(np.float32)
    dev = torch.from_numpy(arr).to("cuda")

    def restore(t):
        return t.cpu().numpy()

    return dev, restore


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def time_integration(primitive_state, config: SimulationConfig, params: SimulationParams,
                     registered_variables: RegisteredVariables, snapshot_callable=None, sharding=None):
    """Integrate to ``params.t_end`` on the GPU (time_integration.py:61-236).

    ``sharding`` is accepted for signature compatibility and ignored: one
    simulation runs on one GPU.
    """
    _check_supported(config)
    if config.state_struct:
        primitive_state = primitive_state.primitive_state
    import torch

    dev, restore = _to_device(primitive_state)
    shape = tuple(dev.shape)
    np_dtype = np.float64 if dev.dtype == torch.float64 else np.float32
    if dev.dtype not in (torch.float32, torch.float64):
        dev = dev.float()
    plan = get_plan(config, registered_variables, shape, np_dtype)
    prm = _native.make_params(params)
    stream = _stream()
    plan.reset(stream)
    ptr = dev.data_ptr()
    huge = 1 << 62
    max_steps = int(config.num_timesteps) if config.fixed_timestep else huge

    if not (config.return_snapshots or config.activate_snapshot_callback):
        info = plan.run(ptr, prm, max_steps, stream)
        _raise_status(info.status, config)
        out = restore(dev)
        return StateStruct(primitive_state=out) if config.state_struct else out

    # ---- snapshots
    n = int(config.num_snapshots)
    ss = config.snapshot_settings
    rec = {"times": [], "states": [], "mass": [], "energy": [], "internal": [], "kinetic": [], "divb": [],
           "radial": [], "grav": []}

    def take(t):
        if config.return_snapshots:
            if len(rec["times"]) >= n:
                return
            rec["times"].append(t)
            if ss.return_states:
                rec["states"].append(restore(dev.clone()))
            sums = plan.conservation_sums(ptr, prm, stream)
            rec["mass"].append(sums[0])
            rec["energy"].append(sums[1])
            rec["kinetic"].append(sums[2])
            rec["internal"].append(sums[3])
            rec["divb"].append(sums[4])
            if config.self_gravity:
                # calculate_total_energy adds 0.5 rho phi (total_quantities.py:141-145)
                eg = _gravitational_energy(dev, config, registered_variables, params, stream)
                rec["energy"][-1] += eg
                rec["grav"].append(eg)
            if ss.return_radial_momentum:
                rec["radial"].append(_radial_momentum(dev, config, registered_variables))
        if config.activate_snapshot_callback and snapshot_callable is not None:
            snapshot_callable(t, restore(dev.clone()), registered_variables)

    steps_taken = 0
    if config.use_specific_snapshot_timepoints and config.return_snapshots:
        # time_integration.py:542-553, :671-678, :742-750: dt is clipped to the
        # next requested time point, a snapshot is taken when t is within
        # 1e-12 of it (at the start of a step), and once more after the step
        # that reaches t_end; the time points are expected to end at t_end
        points = [float(v) for v in np.ravel(np.asarray(params.snapshot_timepoints, dtype=np.float64))]
        k = 0
        t = 0.0
        while True:
            if k < len(points) and abs(t - points[k]) < 1e-12:
                take(t)
                k += 1
            if not (t < params.t_end) or steps_taken >= max_steps:
                break
            target = points[min(k, len(points) - 1)] if points else params.t_end
            if not (target > t):
                target = params.t_end
            info = plan.run(ptr, _native.make_params(params._replace(t_end=target)), max_steps - steps_taken, stream)
            _raise_status(info.status, config)
            steps_taken = info.steps
            t = info.t
            if abs(t - params.t_end) < 1e-12:
                take(t)
                break
    else:
        # pause before the first step starting at t >= k t_end / n
        # (time_integration.py:554-566)
        k = 0
        while True:
            thr = k * params.t_end / n if k < n else math.inf
            info = plan.run_until(ptr, prm, max_steps - steps_taken, thr, stream)
            _raise_status(info.status, config)
            steps_taken = info.steps
            done = (steps_taken >= max_steps) or (not config.fixed_timestep and not (info.t < params.t_end))
            if done:
                break
            take(info.t)
            k += 1
            info = plan.run(ptr, prm, 1, stream)
            _raise_status(info.status, config)
            steps_taken = info.steps
            if steps_taken >= max_steps or (not config.fixed_timestep and not (info.t < params.t_end)):
                break

    final = restore(dev)
    if not config.return_snapshots:
        return StateStruct(primitive_state=final) if config.state_struct else final

    def pad(lst):
        a = np.zeros(n)
        a[:len(lst)] = lst[:n]
        return a

    st = None
    if ss.return_states:
        st = np.zeros((n, *shape), dtype=np_dtype)
        for i, s_ in enumerate(rec["states"][:n]):
            st[i] = np.asarray(s_.cpu() if hasattr(s_, "cpu") else s_)
    return SnapshotData(
        time_points=pad(rec["times"]),
        states=st,
        final_state=final if ss.return_final_state else None,
        total_mass=pad(rec["mass"]) if ss.return_total_mass else None,
        total_energy=pad(rec["energy"]) if ss.return_total_energy else None,
        internal_energy=pad(rec["internal"]) if ss.return_internal_energy else None,
        kinetic_energy=pad(rec["kinetic"]) if ss.return_kinetic_energy else None,
        radial_momentum=pad(rec["radial"]) if ss.return_radial_momentum else None,
        gravitational_energy=pad(rec["grav"]) if (ss.return_gravitational_energy and config.self_gravity) else None,
        magnetic_divergence=pad(rec["divb"]) if (ss.return_magnetic_divergence and config.mhd) else None,
        num_iterations=int(steps_taken),
        current_checkpoint=min(len(rec["times"]), n),
    )


def _radial_momentum(dev, config, rv):
    """calculate_radial_momentum (total_quantities.py:48-71, Cartesian):
    sum of rho u.r_hat dx^d about the box centre, FP64, on the device."""
    import torch

    d = int(config.dimensionality)
    n = dev.shape[-1]
    dx = float(config.grid_spacing)
    x = (torch.arange(n, device=dev.device, dtype=torch.float64) + 0.5) * dx - config.box_size / 2
    grids = torch.meshgrid(*([x] * d), indexing="ij")
    r = torch.sqrt(sum(g * g for g in grids))
    rho = dev[rv.density_index].double()
    ur = sum(dev[1 + i].double() * grids[i] for i in range(d)) / r
    return float((rho * ur).sum() * (dx ** d if d > 1 else dx))


_POISSON = {}


def _poisson(config, n, torch_dtype):
    """The cached Poisson solver of an n^d grid of this config (periodic when
    every boundary is, _poisson_solver.py:39-79)."""
    import torch

    d = int(config.dimensionality)
    lo, hi = _bc_codes(config)
    periodic = all(lo[k] == PERIODIC_BOUNDARY and hi[k] == PERIODIC_BOUNDARY for k in range(d))
    dtype = _native.AMX_F64 if torch_dtype == torch.float64 else _native.AMX_F32
    key = (d, int(n), float(config.grid_spacing), periodic, dtype)
    solver = _POISSON.get(key)
    if solver is None:
        solver = _native.Poisson(d, n, config.grid_spacing, periodic, dtype)
        _POISSON[key] = solver
    return solver


def gravitational_potential(density, config, G=1.0):
    """_compute_gravitational_potential (_poisson_solver.py:17-151) of a CUDA
    tensor of n^d cells on its own grid, on the device."""
    import torch

    rho = density.contiguous()
    phi = torch.empty_like(rho)
    _poisson(config, rho.shape[-1], rho.dtype).solve(rho.data_ptr(), phi.data_ptr(), float(G), _stream())
    return phi


def _gravitational_energy(dev, config, rv, params, stream):
    """calculate_gravitational_energy (total_quantities.py:90-104, Cartesian):
    sum of 0.5 rho phi dx^d, FP64 sum on the device."""
    d = int(config.dimensionality)
    rho = dev[rv.density_index]
    phi = gravitational_potential(rho, config, params.gravitational_constant)
    e = (0.5 * rho.double() * phi.double()).sum()
    return float(e * (config.grid_spacing if d == 1 else config.grid_spacing ** d))


def _raise_status(status, config):
    hard = status & (_native.AMX_ERR_TIMEOUT | _native.AMX_ERR_BOUNDS | _native.AMX_ERR_CUDA)
    if hard:
        raise _native.AmxError(status, "time_integration")
    if config.runtime_debugging and status & (_native.AMX_ERR_NAN | _native.AMX_ERR_NEGATIVE |
                                              _native.AMX_ERR_NOT_CONVERGED):
        raise FloatingPointError(str(_native.AmxError(status, "time_integration")))
