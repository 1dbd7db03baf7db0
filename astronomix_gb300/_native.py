"""ctypes binding of the C ABI declared in include/amx.h.

The library is loaded from ``_lib/libamx.so`` inside this package.  There is
no CPU or eager fallback: if the library is missing, every call raises.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libamx.so")

# ---- error bits (include/amx.h)
AMX_OK = 0
AMX_ERR_INVALID_ARG = 1 << 0
AMX_ERR_CUDA = 1 << 1
AMX_ERR_NAN = 1 << 2
AMX_ERR_NEGATIVE = 1 << 3
AMX_ERR_NOT_CONVERGED = 1 << 4
AMX_ERR_TIMEOUT = 1 << 5
AMX_ERR_BOUNDS = 1 << 6
AMX_ERR_UNSUPPORTED = 1 << 7
AMX_ERR_TOO_LARGE = 1 << 8

_ERR_NAMES = {
    AMX_ERR_INVALID_ARG: "invalid argument",
    AMX_ERR_CUDA: "CUDA runtime error",
    AMX_ERR_NAN: "non-finite value",
    AMX_ERR_NEGATIVE: "negative density or pressure",
    AMX_ERR_NOT_CONVERGED: "magnetic fixed point hit the iteration cap",
    AMX_ERR_TIMEOUT: "grid barrier timed out",
    AMX_ERR_BOUNDS: "index check failed",
    AMX_ERR_UNSUPPORTED: "configuration not supported by the kernels",
    AMX_ERR_TOO_LARGE: "size above a fixed limit",
}

AMX_F32, AMX_F64 = 0, 1


class AmxError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        names = [n for b, n in _ERR_NAMES.items() if code & b]
        super().__init__("%s: %s (code %d)" % (what or "amx", ", ".join(names) or "unknown", code))


class amx_config(ctypes.Structure):
    _fields_ = [
        ("solver_mode", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("dimensionality", ctypes.c_int32),
        ("num_cells", ctypes.c_int32),
        ("num_vars", ctypes.c_int32),
        ("mhd", ctypes.c_int32),
        ("riemann_solver", ctypes.c_int32),
        ("limiter", ctypes.c_int32),
        ("fv_magnetic_integrator", ctypes.c_int32),
        ("numerical_precision", ctypes.c_int32),
        ("boundary_handling", ctypes.c_int32),
        ("bc_lo", ctypes.c_int32 * 3),
        ("bc_hi", ctypes.c_int32 * 3),
        ("enforce_positivity", ctypes.c_int32),
        ("exact_end_time", ctypes.c_int32),
        ("fixed_timestep", ctypes.c_int32),
        ("num_timesteps", ctypes.c_int32),
        ("box_size", ctypes.c_double),
        ("grid_spacing", ctypes.c_double),
        ("split", ctypes.c_int32),
        ("first_order_fallback", ctypes.c_int32),
        ("use_max_adaptive_timestep", ctypes.c_int32),
        ("self_gravity", ctypes.c_int32),
        ("self_gravity_version", ctypes.c_int32),
        ("stellar_wind", ctypes.c_int32),
        ("num_injection_cells", ctypes.c_int32),
        ("turbulent_forcing", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class amx_params(ctypes.Structure):
    _fields_ = [
        ("C_cfl", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("minimum_density", ctypes.c_double),
        ("minimum_pressure", ctypes.c_double),
        ("dt_max", ctypes.c_double),
        ("t_end", ctypes.c_double),
        ("gravitational_constant", ctypes.c_double),
        ("wind_mass_loss_rate", ctypes.c_double),
        ("wind_final_velocity", ctypes.c_double),
        ("energy_injection_rate", ctypes.c_double),
        ("forcing_seed", ctypes.c_int64),
    ]


class amx_run_info(ctypes.Structure):
    _fields_ = [
        ("t", ctypes.c_double),
        ("last_dt", ctypes.c_double),
        ("steps", ctypes.c_int64),
        ("magnetic_iterations", ctypes.c_int64),
        ("last_magnetic_iterations", ctypes.c_int32),
        ("status", ctypes.c_int32),
    ]


_P = ctypes.c_void_p
_D = ctypes.c_double
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64

# name -> (restype, argtypes); the complete list of exports of include/amx.h
SIGNATURES = {
    "amx_plan_create": (_I32, [ctypes.POINTER(amx_config), _I64, ctypes.POINTER(_P)]),
    "amx_plan_destroy": (_I32, [_P]),
    "amx_plan_set_limits": (_I32, [_P, _I32, _I64]),
    "amx_plan_profile": (_I32, [_P, _I32]),
    "amx_plan_profile_read": (_I32, [_P, ctypes.POINTER(_D), ctypes.POINTER(_I64), _I32, _I32]),
    "amx_plan_workspace_bytes": (_I32, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "amx_plan_reset": (_I32, [_P, _P]),
    "amx_plan_set_time": (_I32, [_P, _D, _P]),
    "amx_cfl_dt": (_I32, [_P, _P, ctypes.POINTER(amx_params), ctypes.POINTER(_D), _P]),
    "amx_fv_hydro_rk2": (_I32, [_P, _P, ctypes.POINTER(amx_params), _D, _P]),
    "amx_fv_magnetic_update": (_I32, [_P, _P, ctypes.POINTER(amx_params), _D, _P]),
    "amx_evolve_state": (_I32, [_P, _P, ctypes.POINTER(amx_params), _D, _P]),
    "amx_run": (_I32, [_P, _P, ctypes.POINTER(amx_params), _I64, ctypes.POINTER(amx_run_info), _P]),
    "amx_run_until": (_I32, [_P, _P, ctypes.POINTER(amx_params), _I64, _D, ctypes.POINTER(amx_run_info), _P]),
    "amx_run_async": (_I32, [_P, _P, ctypes.POINTER(amx_params), _I64, _P]),
    "amx_history": (_I32, [_P, ctypes.POINTER(_D), ctypes.POINTER(_I32), _I64, _P]),
    "amx_conservation_sums": (_I32, [_P, _P, ctypes.POINTER(amx_params), ctypes.POINTER(_D), _P]),
    "amx_status": (_I32, [_P, ctypes.POINTER(_I32), _I32, _P]),
    "amx_fv_run_noalloc": (_I32, [ctypes.POINTER(amx_config), _P, ctypes.POINTER(amx_params), _I64,
                                  ctypes.POINTER(amx_run_info), _P]),
    "amx_batch_create": (_I32, [ctypes.POINTER(amx_config), _I32, ctypes.POINTER(_I32), ctypes.POINTER(_D),
                                ctypes.POINTER(_P)]),
    "amx_batch_destroy": (_I32, [_P]),
    "amx_batch_workspace_bytes": (_I32, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "amx_batch_reset": (_I32, [_P, _P]),
    "amx_batch_run": (_I32, [_P, ctypes.POINTER(_P), ctypes.POINTER(amx_params), ctypes.POINTER(_D), _I64, _I32,
                             _P]),
    "amx_batch_info": (_I32, [_P, ctypes.POINTER(amx_run_info), ctypes.POINTER(_I64), _P]),
    "amx_batch_tune": (_I32, [_P, ctypes.POINTER(_P), ctypes.POINTER(amx_params), ctypes.POINTER(_D), _I32,
                              ctypes.POINTER(_D), _P]),
    "amx_batch_tiling": (_I32, [_P, ctypes.POINTER(_I32), ctypes.POINTER(_I32), ctypes.POINTER(_I32),
                                ctypes.POINTER(_I32)]),
    "amx_batch_set_tiling": (_I32, [_P, _I32, _I32]),
    "amx_adjoint_create": (_I32, [ctypes.POINTER(amx_config), _I32, _I64, ctypes.POINTER(_P)]),
    "amx_adjoint_destroy": (_I32, [_P]),
    "amx_adjoint_forward": (_I32, [_P, _P, ctypes.POINTER(amx_params), ctypes.POINTER(amx_run_info), _P]),
    "amx_adjoint_backward": (_I32, [_P, _P, _P, _P]),
    "amx_adjoint_replay": (_I32, [_P, _P, _P]),
    "amx_adjoint_set_tape_budget": (_I32, [_P, ctypes.c_size_t]),
    "amx_adjoint_uses_stored_tape": (_I32, [_P, ctypes.POINTER(_I32)]),
    "amx_adjoint_schedule": (_I32, [_P, ctypes.POINTER(_D), ctypes.POINTER(_I32), _I64, ctypes.POINTER(_I64)]),
    "amx_adjoint_memory": (_I32, [_P, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]),
    "amx_probe_fp32_fma": (_I32, [ctypes.POINTER(_D), _P]),
    "amx_poisson_create": (_I32, [_I32, _I32, _D, _I32, _I32, ctypes.POINTER(_P)]),
    "amx_poisson_destroy": (_I32, [_P]),
    "amx_poisson_solve": (_I32, [_P, _P, _P, _D, _P]),
    "amx_version": (ctypes.c_char_p, []),
}

_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libamx.so not found at %s: build it with `python -m astronomix_gb300._build` "
                "(there is no CPU fallback)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code, what=""):
    if code:
        raise AmxError(code, what)


def make_params(params) -> amx_params:
    return amx_params(
        C_cfl=float(params.C_cfl),
        gamma=float(params.gamma),
        minimum_density=float(params.minimum_density),
        minimum_pressure=float(params.minimum_pressure),
        dt_max=float(params.dt_max),
        t_end=float(params.t_end),
        gravitational_constant=float(getattr(params, "gravitational_constant", 1.0)),
        wind_mass_loss_rate=float(params.wind_params.wind_mass_loss_rate) if hasattr(params, "wind_params") else 0.0,
        wind_final_velocity=float(params.wind_params.wind_final_velocity) if hasattr(params, "wind_params") else 0.0,
        energy_injection_rate=float(params.turbulent_forcing_params.energy_injection_rate)
        if hasattr(params, "turbulent_forcing_params") else 0.0,
        forcing_seed=42,
    )


class Plan:
    """Owns an ``amx_plan`` (device workspace for one configuration)."""

    def __init__(self, cfg: amx_config, max_history: int = 0):
        self._L = lib()
        self.cfg = cfg
        self.max_history = int(max_history)
        h = ctypes.c_void_p()
        check(self._L.amx_plan_create(ctypes.byref(cfg), self.max_history, ctypes.byref(h)), "amx_plan_create")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._L.amx_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    def workspace_bytes(self) -> int:
        n = ctypes.c_size_t()
        check(self._L.amx_plan_workspace_bytes(self.handle, ctypes.byref(n)))
        return n.value

    def set_limits(self, max_fixed_point_iterations=0, barrier_spin_limit=0):
        """Fixed-point cap and grid-barrier poll limit of the FV kernel (0: default)."""
        check(self._L.amx_plan_set_limits(self.handle, int(max_fixed_point_iterations), int(barrier_spin_limit)),
              "amx_plan_set_limits")

    FD_KERNELS = ("cfl", "prep", "weno_x", "weno_y", "weno_z", "emf", "emf_avg", "wind", "update", "finalize",
                  "forcing", "advance")

    def profile(self, enable=True):
        """Per-kernel CUDA-event timing of the FD step (FD plans only)."""
        check(self._L.amx_plan_profile(self.handle, int(bool(enable))), "amx_plan_profile")

    def profile_read(self, reset=True):
        """{kernel kind: (total ms, launches)} since the last reset."""
        n = len(self.FD_KERNELS)
        ms = (ctypes.c_double * n)()
        ln = (ctypes.c_int64 * n)()
        check(self._L.amx_plan_profile_read(self.handle, ms, ln, n, int(bool(reset))), "amx_plan_profile_read")
        return {k: (ms[i], ln[i]) for i, k in enumerate(self.FD_KERNELS)}

    def reset(self, stream=0):
        check(self._L.amx_plan_reset(self.handle, _P(stream)), "amx_plan_reset")

    def set_time(self, t, stream=0):
        check(self._L.amx_plan_set_time(self.handle, float(t), _P(stream)), "amx_plan_set_time")

    def cfl_dt(self, state_ptr, prm: amx_params, stream=0) -> float:
        dt = ctypes.c_double()
        check(self._L.amx_cfl_dt(self.handle, _P(state_ptr), ctypes.byref(prm), ctypes.byref(dt), _P(stream)),
              "amx_cfl_dt")
        return dt.value

    def hydro_rk2(self, state_ptr, prm, dt, stream=0):
        check(self._L.amx_fv_hydro_rk2(self.handle, _P(state_ptr), ctypes.byref(prm), float(dt), _P(stream)),
              "amx_fv_hydro_rk2")

    def magnetic_update(self, state_ptr, prm, dt, stream=0):
        check(self._L.amx_fv_magnetic_update(self.handle, _P(state_ptr), ctypes.byref(prm), float(dt),
                                             _P(stream)), "amx_fv_magnetic_update")

    def evolve(self, state_ptr, prm, dt, stream=0):
        check(self._L.amx_evolve_state(self.handle, _P(state_ptr), ctypes.byref(prm), float(dt), _P(stream)),
              "amx_evolve_state")

    def run(self, state_ptr, prm, max_steps, stream=0) -> amx_run_info:
        info = amx_run_info()
        check(self._L.amx_run(self.handle, _P(state_ptr), ctypes.byref(prm), int(max_steps), ctypes.byref(info),
                              _P(stream)), "amx_run")
        return info

    def run_until(self, state_ptr, prm, max_steps, t_pause, stream=0) -> amx_run_info:
        info = amx_run_info()
        check(self._L.amx_run_until(self.handle, _P(state_ptr), ctypes.byref(prm), int(max_steps), float(t_pause),
                                    ctypes.byref(info), _P(stream)), "amx_run_until")
        return info

    def run_async(self, state_ptr, prm, max_steps, stream=0):
        check(self._L.amx_run_async(self.handle, _P(state_ptr), ctypes.byref(prm), int(max_steps), _P(stream)),
              "amx_run_async")

    def history(self, n, stream=0):
        dts = (ctypes.c_double * n)()
        its = (ctypes.c_int32 * n)()
        check(self._L.amx_history(self.handle, dts, its, int(n), _P(stream)), "amx_history")
        return list(dts), list(its)

    def conservation_sums(self, state_ptr, prm, stream=0):
        out = (ctypes.c_double * 5)()
        check(self._L.amx_conservation_sums(self.handle, _P(state_ptr), ctypes.byref(prm), out, _P(stream)),
              "amx_conservation_sums")
        return list(out)

    def status(self, clear=False, stream=0) -> int:
        st = ctypes.c_int32()
        check(self._L.amx_status(self.handle, ctypes.byref(st), int(bool(clear)), _P(stream)), "amx_status")
        return st.value


class Batch:
    """Owns an ``amx_batch``: device workspace and launch state of an ensemble
    of 2D FV runs sharing one template configuration."""

    def __init__(self, tmpl: amx_config, num_cells, box_size):
        self._L = lib()
        self.num_runs = len(num_cells)
        n = (ctypes.c_int32 * self.num_runs)(*[int(v) for v in num_cells])
        b = (ctypes.c_double * self.num_runs)(*[float(v) for v in box_size])
        h = ctypes.c_void_p()
        check(self._L.amx_batch_create(ctypes.byref(tmpl), self.num_runs, n, b, ctypes.byref(h)), "amx_batch_create")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._L.amx_batch_destroy(h)
            except Exception:
                pass
            self.handle = None

    def _ptrs(self, state_ptrs):
        if len(state_ptrs) != self.num_runs:
            raise ValueError("expected %d state pointers, got %d" % (self.num_runs, len(state_ptrs)))
        return (ctypes.c_void_p * self.num_runs)(*[int(p) for p in state_ptrs])

    def _t_end(self, t_end):
        if len(t_end) != self.num_runs:
            raise ValueError("expected %d end times, got %d" % (self.num_runs, len(t_end)))
        return (ctypes.c_double * self.num_runs)(*[float(t) for t in t_end])

    def workspace_bytes(self) -> int:
        n = ctypes.c_size_t()
        check(self._L.amx_batch_workspace_bytes(self.handle, ctypes.byref(n)))
        return n.value

    def reset(self, stream=0):
        check(self._L.amx_batch_reset(self.handle, _P(stream)), "amx_batch_reset")

    def run(self, state_ptrs, prm: amx_params, t_end, max_steps, use_graph=True, stream=0):
        check(self._L.amx_batch_run(self.handle, self._ptrs(state_ptrs), ctypes.byref(prm), self._t_end(t_end),
                                    int(max_steps), int(bool(use_graph)), _P(stream)), "amx_batch_run")

    def info(self, stream=0):
        infos = (amx_run_info * self.num_runs)()
        lock = ctypes.c_int64()
        check(self._L.amx_batch_info(self.handle, infos, ctypes.byref(lock), _P(stream)), "amx_batch_info")
        return list(infos), lock.value

    def tune(self, state_ptrs, prm: amx_params, t_end, steps=3, stream=0) -> float:
        best = ctypes.c_double()
        check(self._L.amx_batch_tune(self.handle, self._ptrs(state_ptrs), ctypes.byref(prm), self._t_end(t_end),
                                     int(steps), ctypes.byref(best), _P(stream)), "amx_batch_tune")
        return best.value

    def tiling(self):
        v, b, t0, t1 = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        check(self._L.amx_batch_tiling(self.handle, ctypes.byref(v), ctypes.byref(b), ctypes.byref(t0),
                                       ctypes.byref(t1)), "amx_batch_tiling")
        return {"variant": v.value, "blocks_per_sm": b.value, "tile": (t0.value, t1.value)}

    def set_tiling(self, variant, blocks_per_sm=0):
        check(self._L.amx_batch_set_tiling(self.handle, int(variant), int(blocks_per_sm)), "amx_batch_set_tiling")


class Adjoint:
    """Owns an ``amx_adjoint``: checkpoints, schedule and tape of the
    reverse-mode gradient of one FV configuration."""

    def __init__(self, cfg: amx_config, checkpoint_every=20, max_steps=1 << 20):
        self._L = lib()
        h = ctypes.c_void_p()
        check(self._L.amx_adjoint_create(ctypes.byref(cfg), int(checkpoint_every), int(max_steps), ctypes.byref(h)),
              "amx_adjoint_create")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._L.amx_adjoint_destroy(h)
            except Exception:
                pass
            self.handle = None

    def forward(self, state_ptr, prm: amx_params, stream=0) -> amx_run_info:
        info = amx_run_info()
        check(self._L.amx_adjoint_forward(self.handle, _P(state_ptr), ctypes.byref(prm), ctypes.byref(info),
                                          _P(stream)), "amx_adjoint_forward")
        return info

    def backward(self, grad_final_ptr, grad_initial_ptr, stream=0):
        check(self._L.amx_adjoint_backward(self.handle, _P(grad_final_ptr), _P(grad_initial_ptr), _P(stream)),
              "amx_adjoint_backward")

    def set_tape_budget(self, nbytes):
        check(self._L.amx_adjoint_set_tape_budget(self.handle, int(nbytes)), "amx_adjoint_set_tape_budget")

    def uses_stored_tape(self) -> bool:
        y = ctypes.c_int32()
        check(self._L.amx_adjoint_uses_stored_tape(self.handle, ctypes.byref(y)), "amx_adjoint_uses_stored_tape")
        return bool(y.value)

    def replay(self, state_ptr, stream=0):
        check(self._L.amx_adjoint_replay(self.handle, _P(state_ptr), _P(stream)), "amx_adjoint_replay")

    def schedule(self):
        steps = ctypes.c_int64()
        check(self._L.amx_adjoint_schedule(self.handle, None, None, 0, ctypes.byref(steps)), "amx_adjoint_schedule")
        n = steps.value
        dts = (ctypes.c_double * max(n, 1))()
        its = (ctypes.c_int32 * max(n, 1))()
        check(self._L.amx_adjoint_schedule(self.handle, dts, its, n, None), "amx_adjoint_schedule")
        return list(dts)[:n], list(its)[:n]

    def memory(self):
        a, b = ctypes.c_size_t(), ctypes.c_size_t()
        check(self._L.amx_adjoint_memory(self.handle, ctypes.byref(a), ctypes.byref(b)), "amx_adjoint_memory")
        return {"checkpoint_bytes": a.value, "tape_bytes": b.value}


def probe_fp32_fma(stream=0) -> float:
    """Measured FP32 FMA throughput of the current GPU, TFLOP/s."""
    t = ctypes.c_double()
    check(lib().amx_probe_fp32_fma(ctypes.byref(t), _P(stream)), "amx_probe_fp32_fma")
    return t.value


class Poisson:
    """Owns an ``amx_poisson``: the FFT Poisson solve of
    _compute_gravitational_potential on an n^d grid (periodic, or open via
    the Hockney-Eastwood zero padding)."""

    def __init__(self, dimensionality, num_cells, grid_spacing, periodic, dtype):
        self._L = lib()
        h = _P()
        check(self._L.amx_poisson_create(int(dimensionality), int(num_cells), float(grid_spacing), int(bool(periodic)),
                                         int(dtype), ctypes.byref(h)), "amx_poisson_create")
        self.handle = h

    def solve(self, density_ptr, potential_ptr, G, stream=0):
        check(self._L.amx_poisson_solve(self.handle, _P(density_ptr), _P(potential_ptr), float(G), _P(stream)),
              "amx_poisson_solve")

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._L.amx_poisson_destroy(h)
            except Exception:
                pass
            self.handle = None
