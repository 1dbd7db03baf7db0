"""Compiled CPU restatement of the reference's FD step (fd_step.cpp), via ctypes.

TEST INFRASTRUCTURE AND CPU BASELINE ONLY: checked against the NumPy oracle
by the tests and timed by bench.py's CPU legs; the product never imports it.
build() compiles fd_step.cpp with g++ (OpenMP, no floating-point
contraction) into libamxref.so next to this file.
"""
import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fd_step.cpp")
LIB = os.path.join(HERE, "libamxref.so")
FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]

_lib = None


def build(verbose=False):
    """Compiles libamxref.so when it is missing or older than its source."""
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for the CPU restatement")
    tmp = LIB + ".tmp"
    r = subprocess.run([cxx, *FLAGS, SRC, "-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for fd_step.cpp:\n%s" % r.stderr)
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
