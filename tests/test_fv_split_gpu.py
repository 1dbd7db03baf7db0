"""The dimensionally split MUSCL-Hancock FV scheme (config.split = SPLIT,
time_integrator = MUSCL; evolve_state.py:52-325, reconstruction.py:40-129,
_timestep_estimator.py:130-218) through the C ABI against the oracle.

FP64 within 1e-12 of the oracle; FP32 within 1e-5 relative L1 of the FP64
oracle.
"""

import numpy as np
import pytest

import astronomix_gb300 as amx
from astronomix_gb300 import HLL, HLLC, LAX_FRIEDRICHS, AM_HLLC, HYBRID_HLLC, SPLIT, MUSCL, RK2_SSP, DOUBLE_MINMOD
from astronomix_gb300 import OPEN_BOUNDARY, REFLECTIVE_BOUNDARY, PERIODIC_BOUNDARY
from astronomix_gb300 import _native
from astronomix_gb300.time_integration import get_plan
from oracle import driver as odriver, fv as ofv

from _cases import sod, orszag_tang, smooth_random, rel_err, rel_l1

pytestmark = pytest.mark.gpu


def split(cfg, **kw):
    return cfg._replace(split=SPLIT, time_integrator=MUSCL, **kw)


def run_both(cfg, prm, rv, s):
    rec = {}
    ref = odriver.time_integration(s.copy(), cfg, prm, rv, time_mode="float64", record=rec)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    return got, ref, rec


@pytest.mark.parametrize("riemann", [HLL, HLLC, LAX_FRIEDRICHS])
def test_sod_split_fp64(cuda, riemann):
    cfg, prm, rv, s = sod(riemann=riemann, t_end=0.05)
    got, ref, rec = run_both(split(cfg), prm, rv, s)
    assert rec["steps"] > 10
    assert rel_err(got, ref) < 1e-12


@pytest.mark.parametrize("bc", [(REFLECTIVE_BOUNDARY, OPEN_BOUNDARY), (PERIODIC_BOUNDARY, PERIODIC_BOUNDARY)])
def test_sod_split_boundaries_and_limiter_fp64(cuda, bc):
    cfg, prm, rv, s = sod(boundary=bc, limiter=DOUBLE_MINMOD, t_end=0.12)
    got, ref, _ = run_both(split(cfg), prm, rv, s)
    assert rel_err(got, ref) < 1e-12


def test_sod_first_order_fallback_fp64(cuda):
    cfg, prm, rv, s = sod(t_end=0.05)
    cfg = cfg._replace(split=SPLIT, time_integrator=RK2_SSP, first_order_fallback=True)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < 1e-12


def test_sod_split_without_dt_max_clamp(cuda):
    cfg, prm, rv, s = sod(t_end=0.05)
    cfg = split(cfg, use_max_adaptive_timestep=False)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < 1e-12


@pytest.mark.parametrize("dim,n,riemann", [(2, 24, HLLC), (2, 20, LAX_FRIEDRICHS), (3, 10, HLL)])
def test_hydro_split_fp64(cuda, dim, n, riemann):
    cfg, prm, rv, s = smooth_random(dim, n, seed=11, riemann=riemann, t_end=0.02)
    got, ref, rec = run_both(split(cfg), prm, rv, s)
    assert rec["steps"] >= 3
    assert rel_err(got, ref) < 1e-12


@pytest.mark.parametrize("dim,n", [(2, 32), (3, 10)])
def test_mhd_split_fp64(cuda, dim, n):
    if dim == 2:
        cfg, prm, rv, s = orszag_tang(n=n, t_end=0.02)
    else:
        cfg, prm, rv, s = smooth_random(3, n, seed=12, mhd=True, t_end=0.01)
    got, ref, rec = run_both(split(cfg), prm, rv, s)
    assert rec["steps"] >= 3
    assert rel_err(got, ref) < 1e-12


def test_orszag_tang_split_fp32_l1(cuda):
    cfg, prm, rv, s = orszag_tang(n=64, t_end=0.05, dtype=np.float32)
    cfg = split(cfg)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    ref = odriver.time_integration(s.astype(np.float64), cfg, prm, rv, time_mode="float64")
    assert got.dtype == np.float32
    assert rel_l1(got, ref) < 1e-5


def test_split_cfl_seam(cuda):
    import torch

    cfg, prm, rv, s = smooth_random(2, 16, seed=13, riemann=HLLC, t_end=0.02)
    cfg = split(cfg)
    plan = get_plan(cfg, rv, s.shape, np.float64)
    dt = plan.cfl_dt(torch.from_numpy(s).cuda().data_ptr(), _native.make_params(prm),
                     torch.cuda.current_stream().cuda_stream)
    P = ofv.pad(s.copy(), 2)
    P = ofv.boundary_handler(P, cfg)
    ref = ofv.cfl_time_step(P, cfg.grid_spacing, prm.dt_max, prm.gamma, cfg, rv, prm.C_cfl)
    assert dt == pytest.approx(float(ref), rel=1e-15)


# ---- VAN_ALBADA_PP (reconstruction.py:134-394): positivity-preserving
# multidimensional limiting of the unsplit scheme

from astronomix_gb300 import VAN_ALBADA_PP


@pytest.mark.parametrize("dim,n,riemann", [(2, 20, HLLC), (2, 16, LAX_FRIEDRICHS), (3, 10, HLL)])
def test_van_albada_pp_hydro_fp64(cuda, dim, n, riemann):
    cfg, prm, rv, s = smooth_random(dim, n, seed=31, riemann=riemann, limiter=VAN_ALBADA_PP, t_end=0.02)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 3
    assert rel_err(got, ref) < 1e-12


@pytest.mark.parametrize("dim,n", [(2, 32), (3, 10)])
def test_van_albada_pp_mhd_fp64(cuda, dim, n):
    if dim == 2:
        cfg, prm, rv, s = orszag_tang(n=n, t_end=0.02, limiter=VAN_ALBADA_PP)
    else:
        cfg, prm, rv, s = smooth_random(3, n, seed=32, mhd=True, limiter=VAN_ALBADA_PP, t_end=0.03)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 3
    assert rel_err(got, ref) < 1e-12


def test_van_albada_pp_fp32_l1(cuda):
    cfg, prm, rv, s = orszag_tang(n=64, t_end=0.05, dtype=np.float32, limiter=VAN_ALBADA_PP)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    ref = odriver.time_integration(s.astype(np.float64), cfg, prm, rv, time_mode="float64")
    assert rel_l1(got, ref) < 1e-5


def test_van_albada_pp_split_is_van_albada(cuda):
    """The split sweeps use the plain van Albada gradients for VAN_ALBADA_PP
    (limited_gradients.py:72-78; the PP rescaling lives in the unsplit
    reconstruction only)."""
    cfg, prm, rv, s = smooth_random(2, 16, seed=33, riemann=HLLC, limiter=VAN_ALBADA_PP, t_end=0.02)
    got, ref, _ = run_both(split(cfg), prm, rv, s)
    assert rel_err(got, ref) < 1e-12


def test_van_albada_pp_1d_is_rejected(cuda):
    cfg, prm, rv, s = sod(limiter=VAN_ALBADA_PP, t_end=0.01)
    with pytest.raises(_native.AmxError):
        amx.time_integration(s.copy(), cfg, prm, rv)


@pytest.mark.parametrize("dim,n,riemann,boundary", [(2, 24, AM_HLLC, PERIODIC_BOUNDARY),
                                                    (2, 20, HYBRID_HLLC, REFLECTIVE_BOUNDARY),
                                                    (3, 12, AM_HLLC, OPEN_BOUNDARY)])
def test_split_compression_switch_fp64_and_fp32(cuda, dim, n, riemann, boundary):
    """AM_HLLC / HYBRID_HLLC in the split sweeps: the switch of the cell right
    of each face reads its neighbours along every axis of the sweep's input
    (the sweep axis from the staged tile, the others through the boundary
    map).  FP64 within 1e-12 of the oracle, FP32 within 1e-5 relative L1 of
    the FP64 oracle, and the switch changes the result against plain HLLC."""
    cfg, prm, rv, s = smooth_random(dim, n, seed=41, riemann=riemann, boundary=boundary, t_end=0.02, amp=0.5)
    cfg = split(cfg)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 3
    assert rel_err(got, ref) < 1e-12
    plain = odriver.time_integration(s.copy(), cfg._replace(riemann_solver=HLLC), prm, rv, time_mode="float64")
    assert rel_err(plain, ref) > 1e-10
    got32 = amx.time_integration(s.astype(np.float32), cfg, prm, rv)
    for row in range(got32.shape[0]):
        assert rel_l1(got32, ref, row=row) < 1e-5, row
