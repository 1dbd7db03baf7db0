"""The oracle's compiled restatement of the FV step (oracle/cpu/fv_step.cpp)
against the NumPy oracle.

The restatement is the CPU baseline that bench.py times for the FV
workloads; these checks make it a faithful one: FP64 runs of periodic,
unsplit configurations (2D and 3D, hydro and MHD, every restated limiter and
Riemann solver) equal the NumPy oracle with FP64 time to 1e-13, FP32 runs
stay close to FP64, and the thread count does not change the result.
"""
import numpy as np
import pytest

from astronomix_gb300.option_classes import (
    HLL, HLLC, LAX_FRIEDRICHS, MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA)
from oracle import cpu, driver
from _cases import orszag_tang, smooth_random, rel_err, rel_l1


def _pair(cfg, prm, rv, s, max_steps=None):
    rec = {}
    ref = driver.time_integration(np.array(s, dtype=np.float64), cfg, prm, rv, time_mode="float64",
                                  max_steps=max_steps, record=rec)
    x = np.ascontiguousarray(np.array(s, dtype=np.float64))
    t, steps, iters = cpu.fv_run(x, cfg, prm, max_steps=max_steps if max_steps is not None else 1 << 62)
    assert steps == rec["steps"]
    assert t == pytest.approx(rec["t"], rel=1e-14)
    if cfg.mhd:
        assert iters == sum(rec["magnetic_iterations"])
    return x, ref


@pytest.mark.parametrize("riemann", [HLL, HLLC, LAX_FRIEDRICHS])
def test_orszag_tang_2d(riemann):
    cfg, prm, rv, s = orszag_tang(n=32, t_end=0.02, riemann=riemann)
    x, ref = _pair(cfg, prm, rv, s)
    assert rel_err(x, ref) < 1e-13


@pytest.mark.parametrize("limiter", [MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA])
def test_limiters_2d_hydro(limiter):
    cfg, prm, rv, s = smooth_random(2, 24, seed=11 + limiter, limiter=limiter, riemann=HLLC, t_end=0.02)
    x, ref = _pair(cfg, prm, rv, s)
    assert rel_err(x, ref) < 1e-13


@pytest.mark.parametrize("mhd,riemann", [(False, HLLC), (False, LAX_FRIEDRICHS), (True, HLL)])
def test_3d(mhd, riemann):
    cfg, prm, rv, s = smooth_random(3, 12, seed=5, mhd=mhd, riemann=riemann, t_end=0.01)
    x, ref = _pair(cfg, prm, rv, s, max_steps=3)
    assert rel_err(x, ref) < 1e-13


def test_fp32_close_to_fp64():
    cfg, prm, rv, s = orszag_tang(n=32, t_end=0.02)
    x32 = np.ascontiguousarray(s.astype(np.float32))
    x64 = np.ascontiguousarray(s.astype(np.float64))
    cpu.fv_run(x32, cfg, prm)
    cpu.fv_run(x64, cfg, prm)
    assert rel_l1(x32, x64) < 1e-5


def test_threads_do_not_change_results():
    cfg, prm, rv, s = smooth_random(3, 12, seed=9, mhd=True, t_end=0.01)
    a = np.ascontiguousarray(s.copy())
    b = np.ascontiguousarray(s.copy())
    cpu.fv_run(a, cfg, prm, max_steps=2, nthreads=1)
    cpu.fv_run(b, cfg, prm, max_steps=2, nthreads=4)
    assert np.array_equal(a, b)


def test_rejects_unrestated_configurations():
    cfg, prm, rv, s = orszag_tang(n=16, boundary=1)
    with pytest.raises(ValueError):
        cpu.fv_run(np.ascontiguousarray(s.copy()), cfg, prm)
