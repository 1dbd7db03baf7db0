"""Batched ensembles: many independent 2D FV runs in one persistent launch.

The reference integrates one simulation per ``time_integration`` call
(astronomix/time_stepping/time_integration.py:61-236); an ensemble there is
a Python loop over that call.  Here ``time_integration_batched`` hands the
whole ensemble to the C ABI's batch (include/amx.h, amx_batch_*): every run
keeps its own grid size, dt, time and end time, and follows the single-run
kernel bit for bit, while one cooperative launch (optionally replayed from a
CUDA graph) advances all of them.  ``Ensemble.tune`` picks the tile shape and
resident blocks per SM by timing trial steps on copies of the states.

The initial conditions of the turbulent ensemble come from
``create_turb_field``, a NumPy restatement of the reference's Gaussian random
field generator (astronomix/initial_condition_generation/
turbulent_ic_generator.py:19-109) extended to 2D.
"""

from typing import List, Sequence

import numpy as np

from . import _native
from .option_classes import (
    SimulationConfig, SimulationParams, BoundarySettings, BoundarySettings1D, finalize_config,
    FINITE_VOLUME, HLLC, MINMOD, PERIODIC_BOUNDARY, DOUBLE_PRECISION, SINGLE_PRECISION,
)
from .variable_registry import get_registered_variables, RegisteredVariables
from .setup_helpers import construct_primitive_state
from .time_integration import make_amx_config, _check_supported, _stream, _raise_status

__all__ = ["create_turb_field", "turbulent_ensemble_member", "Ensemble", "time_integration_batched"]


# ------------------------------------------------------------------ initial conditions

def _cosine_taper(k, k0, k1):
    """1 for k <= k0, a half cosine down to 0 at k1 (turbulent_ic_generator.py:5-14)."""
    if k1 <= k0 + 1e-12:
        return np.where(k <= k0, 1.0, 0.0)
    t = np.clip((k - k0) / (k1 - k0), 0.0, 1.0)
    return np.where(k <= k0, 1.0, 0.5 * (1.0 + np.cos(np.pi * t)))


def create_turb_field(Ndim, A0, slope, kmin, kmax, seed=0, dimensionality=3, kroll_frac=0.85, zero_mean=True,
                      rng=None):
    """Real Gaussian random field on an Ndim^d periodic grid whose Fourier
    amplitude scales as A0 * |k|^slope inside kmin <= |k| <= kmax, with a
    cosine roll-off from kroll_frac * kmax (turbulent_ic_generator.py:19-109).

    The complex coefficients are normal with standard deviation
    amplitude / sqrt(2) per part, made Hermitian by averaging with the
    conjugate at -k, real at the self-conjugate modes, and the field is the
    real part of the inverse FFT.  Random numbers come from NumPy's
    ``default_rng(seed)`` (or ``rng``) instead of jax.random, so a seed gives
    a different (equally distributed) field than the reference's key.
    """
    if dimensionality not in (1, 2, 3):
        raise ValueError("dimensionality must be 1, 2 or 3")
    rng = np.random.default_rng(seed) if rng is None else rng
    k1d = np.fft.fftfreq(Ndim, d=1.0) * Ndim
    shape = (Ndim,) * dimensionality
    ksq = np.zeros(shape)
    for ax in range(dimensionality):
        view = [1] * dimensionality
        view[ax] = Ndim
        ksq = ksq + k1d.reshape(view) ** 2
    k = np.sqrt(ksq)
    taper = _cosine_taper(k, kroll_frac * kmax, kmax)
    band = (k >= kmin) & (k <= kmax)
    k_safe = np.where(k == 0.0, 1.0, k)
    amp = A0 * k_safe ** slope
    if zero_mean:
        amp[(0,) * dimensionality] = 0.0
    amp = amp * band * taper
    sigma = amp / np.sqrt(2.0)
    F = rng.standard_normal(shape) * sigma + 1j * (rng.standard_normal(shape) * sigma)
    axes = tuple(range(dimensionality))
    F_neg = np.roll(np.flip(np.conj(F), axis=axes), shift=1, axis=axes)  # conj(F(-k))
    F = 0.5 * (F + F_neg)
    idx = np.arange(Ndim)
    sc = idx == ((-idx) % Ndim)
    self_conj = np.ones(shape, dtype=bool)
    for ax in range(dimensionality):
        view = [1] * dimensionality
        view[ax] = Ndim
        self_conj = self_conj & sc.reshape(view)
    F = np.where(self_conj, F.real + 0j, F)
    if zero_mean:
        F[(0,) * dimensionality] = 0.0
    return np.real(np.fft.ifftn(F))


ENSEMBLE_SIZES = (128, 192, 256, 384, 512)


def turbulent_ensemble_member(seed, sizes=ENSEMBLE_SIZES, t_end_range=(0.05, 0.2), gamma=5.0 / 3.0, mach=1.0,
                              beta=1.0, k_max=44, C_cfl=0.4, dtype=np.float32, size_override=None):
    """One run of the turbulent 2D MHD ensemble, drawn from ``default_rng(seed)``:
    grid size N uniform from ``sizes`` on the unit periodic box, t_end uniform
    in ``t_end_range``, velocity a 2D Gaussian random field per component with
    Fourier amplitude ~ k^-2 (per-mode power ~ k^-4) on 1 <= k <= k_max scaled
    to rms Mach ``mach`` (v_rms = mach * sqrt(gamma p / rho)), rho = 1, p = 1,
    uniform B_x = sqrt(2 p / beta); FV HLLC, MINMOD, implicit-midpoint
    magnetic update.  Returns (config, params, registered_variables, state).
    ``size_override`` replaces the drawn N (small test ensembles)."""
    rng = np.random.default_rng(seed)
    n = int(rng.choice(np.asarray(sizes)))
    t_end = float(rng.uniform(*t_end_range))
    if size_override is not None:
        n = int(size_override)
    kmax = min(float(k_max), 0.7 * n / 2)
    vx = create_turb_field(n, 1.0, -2.0, 1.0, kmax, dimensionality=2, rng=rng)
    vy = create_turb_field(n, 1.0, -2.0, 1.0, kmax, dimensionality=2, rng=rng)
    rho, p = 1.0, 1.0
    cs = np.sqrt(gamma * p / rho)
    rms = np.sqrt(np.mean(vx ** 2 + vy ** 2))
    scale = mach * cs / rms
    vx, vy = vx * scale, vy * scale
    cfg = SimulationConfig(
        mhd=True, dimensionality=2, box_size=1.0, num_cells=n, riemann_solver=HLLC, limiter=MINMOD,
        numerical_precision=DOUBLE_PRECISION if np.dtype(dtype) == np.float64 else SINGLE_PRECISION,
        boundary_settings=BoundarySettings(*[BoundarySettings1D(PERIODIC_BOUNDARY, PERIODIC_BOUNDARY)] * 3))
    rv = get_registered_variables(cfg)
    ones = np.ones((n, n))
    bx = np.sqrt(2.0 * p / beta)
    state = construct_primitive_state(cfg, rv, density=rho * ones, velocity_x=vx, velocity_y=vy,
                                      gas_pressure=p * ones, magnetic_field_x=bx * ones,
                                      magnetic_field_y=0.0 * ones, magnetic_field_z=0.0 * ones)
    state = np.asarray(state, dtype=dtype)
    cfg = finalize_config(cfg, state.shape)
    prm = SimulationParams(t_end=t_end, gamma=gamma, C_cfl=C_cfl)
    return cfg, prm, rv, state


# ------------------------------------------------------------------ the batch

_SHARED_FIELDS = [f for f, _ in _native.amx_config._fields_ if f not in ("num_cells", "box_size", "grid_spacing")]
_PARAM_FIELDS = ("C_cfl", "gamma", "minimum_density", "minimum_pressure", "dt_max")


def _template(configs, registered_variables, shapes, dtype):
    cs = [make_amx_config(c, registered_variables, s, dtype) for c, s in zip(configs, shapes)]
    t = cs[0]
    for i, c in enumerate(cs[1:], 1):
        for f in _SHARED_FIELDS:
            a, b = getattr(t, f), getattr(c, f)
            if hasattr(a, "__len__"):
                a, b = list(a), list(b)
            if a != b:
                raise ValueError("run %d differs from run 0 in %s: a batch shares everything but the grid "
                                 "size, the box size and t_end" % (i, f))
    for c, s in zip(configs, shapes):
        if s[-1] != s[-2]:
            raise ValueError("batched runs are square 2D grids")
    return t, cs


class Ensemble:
    """A device-resident ensemble of 2D FV runs sharing one configuration
    template (everything except grid size, box size and ``t_end``)."""

    def __init__(self, configs: Sequence[SimulationConfig], params: Sequence[SimulationParams],
                 registered_variables: RegisteredVariables, shapes, dtype=np.float32):
        if len(configs) != len(params) or len(configs) != len(shapes):
            raise ValueError("configs, params and shapes must have one entry per run")
        for c in configs:
            _check_supported(c)
            if c.solver_mode != FINITE_VOLUME or c.dimensionality != 2:
                raise NotImplementedError("batched runs are 2D finite-volume runs")
        p0 = params[0]
        for i, p in enumerate(params[1:], 1):
            for f in _PARAM_FIELDS:
                if float(getattr(p, f)) != float(getattr(p0, f)):
                    raise ValueError("run %d differs from run 0 in params.%s" % (i, f))
        self.dtype = np.dtype(dtype)
        self.tmpl, self.cfgs = _template(configs, registered_variables, shapes, self.dtype)
        self.configs = list(configs)
        self.registered_variables = registered_variables
        self.shapes = [tuple(s) for s in shapes]
        self.t_end = [float(p.t_end) for p in params]
        self.prm = _native.make_params(p0)
        self.batch = _native.Batch(self.tmpl, [c.num_cells for c in self.cfgs], [c.box_size for c in self.cfgs])

    @property
    def num_runs(self):
        return len(self.shapes)

    def _ptrs(self, states):
        import torch

        ptrs = []
        want = torch.float64 if self.dtype == np.float64 else torch.float32
        for s, shp in zip(states, self.shapes):
            if not (isinstance(s, torch.Tensor) and s.is_cuda and s.is_contiguous() and s.dtype == want and
                    tuple(s.shape) == shp):
                raise ValueError("ensemble states must be contiguous CUDA tensors of shape %s and %s" % (shp, want))
            ptrs.append(s.data_ptr())
        return ptrs

    def reset(self):
        self.batch.reset(_stream())

    def tune(self, states, steps=3) -> dict:
        """Times ``steps`` lock-step steps per tile shape / resident-block
        count on copies of ``states`` and keeps the fastest."""
        best = self.batch.tune(self._ptrs(states), self.prm, self.t_end, steps, _stream())
        out = self.batch.tiling()
        out["trial_ms"] = best
        return out

    def run(self, states, max_steps=None, use_graph=True):
        """Advances the device tensors ``states`` in place (asynchronous)."""
        ms = (1 << 62) if max_steps is None else int(max_steps)
        self.batch.run(self._ptrs(states), self.prm, self.t_end, ms, use_graph, _stream())

    def info(self):
        """(list of amx_run_info, lock-step steps taken); synchronises."""
        return self.batch.info(_stream())


def time_integration_batched(initial_states: Sequence, configs: Sequence[SimulationConfig],
                             params: Sequence[SimulationParams], registered_variables: RegisteredVariables,
                             tune: bool = False, use_graph: bool = True, return_info: bool = False):
    """``time_integration`` for a list of independent 2D FV runs at once.

    Run i is ``time_integration(initial_states[i], configs[i], params[i],
    registered_variables)`` (final state only): same result, computed by one
    persistent launch for the whole ensemble.  States may be NumPy arrays or
    torch tensors (one dtype for all); results come back in the same form.
    """
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("astronomix_gb300 runs on a CUDA GPU; no device is visible")
    devs, restores = [], []
    dtype = None
    for s in initial_states:
        if isinstance(s, torch.Tensor):
            d = s.detach().to("cuda").contiguous().clone()
            restores.append((lambda was_cuda: (lambda t: t if was_cuda else t.cpu()))(s.is_cuda))
        else:
            a = np.ascontiguousarray(s)
            if a.dtype not in (np.float32, np.float64):
                a = a.astype(np.float32)
            d = torch.from_numpy(a).to("cuda")
            restores.append(lambda t: t.cpu().numpy())
        dt_ = np.float64 if d.dtype == torch.float64 else np.float32
        if dtype is None:
            dtype = dt_
        elif dtype != dt_:
            raise ValueError("all ensemble states must share one dtype")
        devs.append(d)
    ens = Ensemble(configs, params, registered_variables, [tuple(d.shape) for d in devs], dtype)
    if tune:
        ens.tune(devs)
    ens.run(devs, use_graph=use_graph)
    infos, lock = ens.info()
    for i, c in zip(infos, configs):
        _raise_status(i.status, c)
    outs = [r(d) for r, d in zip(restores, devs)]
    if return_info:
        return outs, infos
    return outs
