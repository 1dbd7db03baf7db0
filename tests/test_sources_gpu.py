"""The FD source hooks through the C ABI against the oracle: the stellar-wind
EI source in every SSPRK stage's right-hand side (_ssprk.py:230-241,
stellar_wind.py:485-584) and the turbulent forcing before every step
(_turbulent_forcing.py:15-128, time_integration.py:700-711), for the FD
scheme and for the FV scheme with periodic roll.

FP64 to 1e-11 of the oracle (the forcing field comes out of an inverse FFT:
cuFFT and NumPy's pocketfft round differently at 1e-16); FP32 within 1e-5
relative L1 of the FP64 oracle.  The forcing's random stream is the Philox
generator both sides share (oracle/forcing.py).
"""

import numpy as np
import pytest

import astronomix_gb300 as amx
from astronomix_gb300 import PERIODIC_BOUNDARY, HLL, HLLC
from astronomix_gb300.option_classes import WindConfig, WindParams, TurbulentForcingConfig, TurbulentForcingParams
from oracle import driver as odriver

from _cases import blast_fd, smooth_random, rel_err, rel_l1

pytestmark = pytest.mark.gpu

TOL = 1e-11
# no field component zero: with B_n = 0 the reference's eigenvectors are
# ill-conditioned (a 1e-15 perturbation moves its result by 1e-8)
OBLIQUE = (0.6, 0.5, 0.4)


def with_wind(cfg, prm, nic=3, mdot=2.0, vinf=3.0):
    cfg = cfg._replace(wind_config=WindConfig(stellar_wind=True, num_injection_cells=nic))
    prm = prm._replace(wind_params=WindParams(wind_mass_loss_rate=mdot, wind_final_velocity=vinf))
    return cfg, prm


def with_forcing(cfg, prm, edot=20.0):
    cfg = cfg._replace(turbulent_forcing_config=TurbulentForcingConfig(turbulent_forcing=True))
    prm = prm._replace(turbulent_forcing_params=TurbulentForcingParams(energy_injection_rate=edot))
    return cfg, prm


def run_both(cfg, prm, rv, s):
    rec = {}
    ref = odriver.time_integration(s.astype(np.float64), cfg, prm, rv, time_mode="float64", record=rec)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    return got, ref, rec


def test_fd_stellar_wind_fp64(cuda):
    cfg, prm, rv, s = blast_fd(n=16, t_end=0.004, B=OBLIQUE)
    cfg, prm = with_wind(cfg, prm)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 3
    assert rel_err(got, ref) < TOL
    plain = amx.time_integration(s.copy(), cfg._replace(wind_config=WindConfig()), prm, rv)
    assert np.abs(got[0] - plain[0]).max() > 1e-4  # the source acts


def test_fd_turbulent_forcing_fp64(cuda):
    cfg, prm, rv, s = blast_fd(n=16, t_end=0.004, B=OBLIQUE)
    cfg, prm = with_forcing(cfg, prm)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 3
    assert rel_err(got, ref) < TOL
    plain = amx.time_integration(s.copy(), cfg._replace(turbulent_forcing_config=TurbulentForcingConfig()), prm, rv)
    assert np.abs(got[1] - plain[1]).max() > 1e-4


def test_fd_wind_and_forcing_fp64(cuda):
    """The showcase combination: driven turbulence with a wind source."""
    cfg, prm, rv, s = blast_fd(n=24, t_end=0.0015, B=OBLIQUE)
    cfg, prm = with_wind(cfg, prm, nic=4)
    cfg, prm = with_forcing(cfg, prm)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < TOL


def test_fd_wind_and_forcing_fp32(cuda):
    cfg, prm, rv, s = blast_fd(n=24, dtype=np.float32, t_end=0.0015, B=OBLIQUE)
    cfg, prm = with_wind(cfg, prm, nic=4)
    cfg, prm = with_forcing(cfg, prm)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert got.dtype == np.float32
    assert rel_l1(got, ref) < 1e-5
    assert rel_l1(got, ref, row=1) < 1e-4


@pytest.mark.parametrize("mhd", [False, True])
def test_fv_turbulent_forcing_roll_fp64(cuda, mhd):
    cfg, prm, rv, s = smooth_random(3, 16, seed=4, mhd=mhd, riemann=HLL if mhd else HLLC, roll=True, t_end=0.01)
    cfg, prm = with_forcing(cfg, prm, edot=5.0)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 3
    assert rel_err(got, ref) < TOL


def test_forcing_rejected_with_ghost_cells(cuda):
    cfg, prm, rv, s = smooth_random(3, 12, seed=4, roll=False, t_end=0.01)
    cfg, prm = with_forcing(cfg, prm)
    with pytest.raises(ValueError):
        amx.time_integration(s.copy(), cfg, prm, rv)


def test_fv_forcing_with_snapshot_pauses_fp64(cuda):
    """Pausing at snapshot times (amx_run_until on the device-driven steps)
    leaves the forced run's result unchanged."""
    from astronomix_gb300 import SnapshotSettings

    cfg, prm, rv, s = smooth_random(3, 12, seed=5, riemann=HLLC, roll=True, t_end=0.012)
    cfg, prm = with_forcing(cfg, prm, edot=5.0)
    ref = odriver.time_integration(s.copy(), cfg, prm, rv, time_mode="float64")
    cfg = cfg._replace(return_snapshots=True, num_snapshots=3,
                       snapshot_settings=SnapshotSettings(return_final_state=True, return_total_energy=True))
    snap = amx.time_integration(s.copy(), cfg, prm, rv)
    assert rel_err(snap.final_state, ref) < TOL
    assert snap.num_iterations >= 3
