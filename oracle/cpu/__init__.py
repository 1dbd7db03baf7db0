"""Compiled CPU restatements of the reference's FD step (fd_step.cpp) and FV
step (fv_step.cpp), via ctypes.

TEST INFRASTRUCTURE AND CPU BASELINE ONLY: checked against the NumPy oracle
by the tests and timed by bench.py's CPU legs; the product never imports it.
build() compiles both sources with g++ (OpenMP, no floating-point
contraction) into libamxref.so next to this file.
"""
import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "fd_step.cpp"), os.path.join(HERE, "fv_step.cpp")]
LIB = os.path.join(HERE, "libamxref.so")
FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]

_lib = None


def build(verbose=False):
    """Compiles libamxref.so when it is missing or older than its source."""
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in SRCS):
        return LIB
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for the CPU restatement")
    tmp = LIB + ".tmp"
    r = subprocess.run([cxx, *FLAGS, *SRCS, "-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for the CPU restatement:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.amxref_fd_run.restype = ctypes.c_int
        L.amxref_fd_run.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 7 + [
            ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
            ctypes.POINTER(ctypes.c_int64), ctypes.c_int]
        L.amxref_fv_run.restype = ctypes.c_int
        L.amxref_fv_run.argtypes = [ctypes.c_int] * 7 + [ctypes.c_double] * 5 + [
            ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
            ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64), ctypes.c_int]
        L.amxref_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def threads():
    return lib().amxref_threads()


def fd_run(state, config, params, max_steps=1 << 62, nthreads=0):
    """Advances a float32/float64 NumPy FD state (11 x n^3, C order) in place,
    like the reference's time_integration of an FD configuration, for at most
    max_steps steps.  Returns (t, steps)."""
    import numpy as np

    assert state.flags["C_CONTIGUOUS"] and state.dtype in (np.float32, np.float64)
    n = state.shape[-1]
    t = ctypes.c_double()
    steps = ctypes.c_int64()
    rc = lib().amxref_fd_run(0 if state.dtype == np.float32 else 1, n, float(config.grid_spacing),
                             float(params.gamma), float(params.minimum_density), float(params.minimum_pressure),
                             float(params.C_cfl), float(params.dt_max), float(params.t_end),
                             int(bool(config.exact_end_time)), int(bool(config.enforce_positivity)),
                             int(max_steps), state.ctypes.data, ctypes.byref(t), ctypes.byref(steps), int(nthreads))
    if rc:
        raise RuntimeError("amxref_fd_run failed (%d)" % rc)
    return t.value, steps.value


def fv_run(state, config, params, max_steps=1 << 62, nthreads=0):
    """Advances a float32/float64 NumPy FV state (nv x n^dim, C order) in
    place like the reference's time_integration of an unsplit, periodic FV
    configuration (FP64 time and dt), for at most max_steps steps.  Returns
    (t, steps, fixed-point iterations)."""
    import numpy as np
    from astronomix_gb300.option_classes import (
        FINITE_VOLUME, UNSPLIT, HLL, HLLC, LAX_FRIEDRICHS, MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA,
        IMPLICIT_MIDPOINT, SINGLE_PRECISION, PERIODIC_BOUNDARY, PERIODIC_ROLL)

    assert state.flags["C_CONTIGUOUS"] and state.dtype in (np.float32, np.float64)
    if config.solver_mode != FINITE_VOLUME or config.split != UNSPLIT:
        raise ValueError("the FV restatement covers the unsplit finite-volume scheme")
    if config.riemann_solver not in (HLL, HLLC, LAX_FRIEDRICHS):
        raise ValueError("Riemann solver %d is not restated" % config.riemann_solver)
    if config.limiter not in (MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA):
        raise ValueError("limiter %d is not restated" % config.limiter)
    if config.boundary_handling != PERIODIC_ROLL:
        bs = config.boundary_settings
        sides = [bs.x, bs.y] + ([bs.z] if config.dimensionality == 3 else [])
        if any(s.left_boundary != PERIODIC_BOUNDARY or s.right_boundary != PERIODIC_BOUNDARY for s in sides):
            raise ValueError("the FV restatement covers periodic boundaries")
    n = state.shape[-1]
    t = ctypes.c_double()
    steps = ctypes.c_int64()
    iters = ctypes.c_int64()
    tol = 1e-5 if config.numerical_precision == SINGLE_PRECISION else 1e-10
    rc = lib().amxref_fv_run(0 if state.dtype == np.float32 else 1, int(config.dimensionality), n,
                             int(bool(config.mhd)), int(config.limiter), int(config.riemann_solver),
                             int(config.fv_magnetic_integrator == IMPLICIT_MIDPOINT), float(config.grid_spacing),
                             float(params.gamma), float(params.C_cfl), float(params.t_end), tol,
                             int(bool(config.exact_end_time)), int(max_steps), state.ctypes.data,
                             ctypes.byref(t), ctypes.byref(steps), ctypes.byref(iters), int(nthreads))
    if rc:
        raise RuntimeError("amxref_fv_run failed (%d)" % rc)
    return t.value, steps.value, iters.value
