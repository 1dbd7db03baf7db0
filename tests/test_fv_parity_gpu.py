"""Finite-volume CUDA path vs the oracle (reference restatement), through the C ABI.

FP64: every field within 1e-12 of the oracle, relative to the field's scale.
FP32: relative L1 density error within 1e-5 of the FP32 oracle and of the
FP64 oracle (the tolerance of the benchmark metric).
"""

import numpy as np
import pytest

import astronomix_gb300 as amx
from astronomix_gb300 import HLL, HLLC, HLLC_LM, LAX_FRIEDRICHS, MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA
from astronomix_gb300 import OPEN_BOUNDARY, REFLECTIVE_BOUNDARY, PERIODIC_BOUNDARY
from oracle import driver as odriver

from _cases import sod, orszag_tang, smooth_random, rel_err, rel_l1

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def run_both(cfg, prm, rv, s, time_mode="reference"):
    rec = {}
    ref = odriver.time_integration(s.copy(), cfg, prm, rv, time_mode=time_mode, record=rec)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    return got, ref, rec


@pytest.mark.parametrize("riemann", [HLL, HLLC, HLLC_LM, LAX_FRIEDRICHS])
def test_sod_fp64_matches_oracle(cuda, riemann):
    cfg, prm, rv, s = sod(riemann=riemann, t_end=0.05)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] > 5
    assert rel_err(got, ref) < FP64_TOL


@pytest.mark.parametrize("limiter", [MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA])
def test_sod_limiters_fp64(cuda, limiter):
    cfg, prm, rv, s = sod(limiter=limiter, t_end=0.03)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < FP64_TOL


@pytest.mark.parametrize("bc", [(REFLECTIVE_BOUNDARY, REFLECTIVE_BOUNDARY), (PERIODIC_BOUNDARY, PERIODIC_BOUNDARY),
                                (REFLECTIVE_BOUNDARY, OPEN_BOUNDARY)])
def test_sod_boundaries_fp64(cuda, bc):
    cfg, prm, rv, s = sod(boundary=bc, t_end=0.15)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < FP64_TOL


def test_sod_full_fp32_vs_fp64(cuda):
    cfg, prm, rv, s = sod(dtype=np.float32)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    ref32 = odriver.time_integration(s.copy(), cfg, prm, rv, time_mode="float64")
    ref64 = odriver.time_integration(s.astype(np.float64), cfg, prm, rv)
    assert got.dtype == np.float32
    assert rel_l1(got, ref32) < 1e-5
    assert rel_l1(got, ref64) < 1e-5


@pytest.mark.parametrize("riemann", [HLL, HLLC, LAX_FRIEDRICHS])
@pytest.mark.parametrize("dim", [2, 3])
def test_hydro_periodic_fp64(cuda, dim, riemann):
    n = 24 if dim == 2 else 12
    cfg, prm, rv, s = smooth_random(dim, n, seed=dim * 10 + riemann, riemann=riemann, t_end=0.01)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 2
    assert rel_err(got, ref) < FP64_TOL


@pytest.mark.parametrize("boundary", [OPEN_BOUNDARY, REFLECTIVE_BOUNDARY])
def test_hydro_2d_nonperiodic_fp64(cuda, boundary):
    cfg, prm, rv, s = smooth_random(2, 20, seed=7, boundary=boundary, t_end=0.01)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < FP64_TOL


@pytest.mark.parametrize("roll", [False, True])
@pytest.mark.parametrize("riemann", [HLL, HLLC])
def test_orszag_tang_fp64(cuda, roll, riemann):
    cfg, prm, rv, s = orszag_tang(n=48, t_end=0.01, roll=roll, riemann=riemann)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 5
    assert rel_err(got, ref) < FP64_TOL


@pytest.mark.parametrize("riemann", [HLL, LAX_FRIEDRICHS])
def test_mhd_3d_fp64(cuda, riemann):
    cfg, prm, rv, s = smooth_random(3, 12, seed=3, mhd=True, riemann=riemann, t_end=0.005)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 2
    assert rel_err(got, ref) < FP64_TOL


def test_orszag_tang_fp32_l1(cuda):
    cfg, prm, rv, s = orszag_tang(n=64, t_end=0.05, dtype=np.float32)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    ref64 = odriver.time_integration(s.astype(np.float64), cfg, prm, rv)
    assert got.dtype == np.float32
    assert rel_l1(got, ref64) < 1e-5
