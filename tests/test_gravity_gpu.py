"""Self-gravity (_physics_modules/_self_gravity/*) through the C ABI against the oracle.

The Poisson solve (amx_poisson_solve: periodic FFT and the Hockney-Eastwood
open-boundary convolution, 1D/2D/3D) to 1e-12 of the oracle's NumPy FFT
solve in FP64; runs with the source term of every version, unsplit and
split, hydro and MHD, ghost-cell and periodic-roll handling, periodic, open
and reflective boundaries to 1e-11 in FP64 (cuFFT and NumPy's FFT round
differently: the potential differs at 1e-16 relative, the accelerations,
differences of it over one cell, at about n times that); FP32 within 1e-5
relative L1 of the FP64 oracle.
"""

import numpy as np
import pytest

import astronomix_gb300 as amx
from astronomix_gb300 import (
    HLL, HLLC, HLLC_LM, LAX_FRIEDRICHS, AM_HLLC, HYBRID_HLLC, SPLIT, MUSCL, RK2_SSP, OPEN_BOUNDARY, REFLECTIVE_BOUNDARY,
    PERIODIC_BOUNDARY,
    SIMPLE_SOURCE_TERM, DONOR_ACCOUNTING, RIEMANN_SPLIT, RIEMANN_SPLIT_UNSTABLE, HALF_SPLIT, _native,
)
from oracle import driver as odriver, gravity as ograv

from _cases import smooth_random, rel_err, rel_l1

pytestmark = pytest.mark.gpu

TOL = 1e-11


def grav_case(dim, n, version=DONOR_ACCOUNTING, riemann=HLL, boundary=PERIODIC_BOUNDARY, split=False, mhd=False,
              roll=False, dtype=np.float64, t_end=0.02, G=2.0, seed=3, first_order=False):
    cfg, prm, rv, s = smooth_random(dim, n, seed=seed, dtype=dtype, mhd=mhd, riemann=riemann, boundary=boundary,
                                    roll=roll, t_end=t_end)
    cfg = cfg._replace(self_gravity=True, self_gravity_version=version)
    if split:
        cfg = cfg._replace(split=SPLIT, time_integrator=MUSCL)
    if first_order:
        cfg = cfg._replace(split=SPLIT, time_integrator=RK2_SSP, first_order_fallback=True)
    prm = prm._replace(gravitational_constant=G)
    return cfg, prm, rv, s


def run_both(cfg, prm, rv, s):
    rec = {}
    ref = odriver.time_integration(s.astype(np.float64), cfg, prm, rv, time_mode="float64", record=rec)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    return got, ref, rec


def _bcfg(dim, boundary, dx=1.0 / 32):
    from types import SimpleNamespace
    from astronomix_gb300 import BoundarySettings, BoundarySettings1D

    b = BoundarySettings1D(boundary, boundary)
    bs = b if dim == 1 else BoundarySettings(b, b, b)
    return SimpleNamespace(dimensionality=dim, boundary_settings=bs, grid_spacing=dx)


@pytest.mark.parametrize("dim,n", [(1, 64), (2, 48), (3, 20)])
@pytest.mark.parametrize("boundary", [PERIODIC_BOUNDARY, OPEN_BOUNDARY])
def test_poisson_solve_fp64(cuda, dim, n, boundary):
    import torch

    rng = np.random.default_rng(dim * 7 + n)
    rho = 1.0 + 0.3 * rng.random((n,) * dim)
    cfg = _bcfg(dim, boundary, dx=1.0 / n)
    ref = ograv.gravitational_potential(rho, cfg.grid_spacing, cfg, 1.7)
    got = amx.gravitational_potential(torch.from_numpy(rho).cuda(), cfg, 1.7).cpu().numpy()
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-12


@pytest.mark.parametrize("boundary", [PERIODIC_BOUNDARY, OPEN_BOUNDARY])
def test_poisson_solve_fp32(cuda, boundary):
    import torch

    n = 64
    rng = np.random.default_rng(5)
    rho = 1.0 + 0.3 * rng.random((n, n))
    cfg = _bcfg(2, boundary, dx=1.0 / n)
    ref = ograv.gravitational_potential(rho, cfg.grid_spacing, cfg, 1.0)
    got = amx.gravitational_potential(torch.from_numpy(rho.astype(np.float32)).cuda(), cfg, 1.0).cpu().numpy()
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-5


def test_poisson_periodic_analytic(cuda):
    """lap(phi) = 4 pi G (rho - mean): a single Fourier mode has phi = -4 pi G A sin(kx) / k^2."""
    import torch

    n = 64
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    rho = 1.0 + 0.1 * np.sin(2 * np.pi * X)
    cfg = _bcfg(2, PERIODIC_BOUNDARY, dx=1.0 / n)
    got = amx.gravitational_potential(torch.from_numpy(rho).cuda(), cfg, 1.0).cpu().numpy()
    exact = -4 * np.pi * 0.1 * np.sin(2 * np.pi * X) / (2 * np.pi) ** 2
    assert np.abs(got - exact).max() < 1e-12


@pytest.mark.parametrize("version", [SIMPLE_SOURCE_TERM, DONOR_ACCOUNTING, HALF_SPLIT])
@pytest.mark.parametrize("riemann", [HLL, HLLC, LAX_FRIEDRICHS])
def test_unsplit_2d_periodic_versions_fp64(cuda, version, riemann):
    cfg, prm, rv, s = grav_case(2, 24, version=version, riemann=riemann)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 4
    assert rel_err(got, ref) < TOL


@pytest.mark.parametrize("version", [SIMPLE_SOURCE_TERM, DONOR_ACCOUNTING, HALF_SPLIT])
@pytest.mark.parametrize("riemann", [AM_HLLC, HYBRID_HLLC])
def test_compression_switch_versions_fp64(cuda, version, riemann):
    """AM_HLLC / HYBRID_HLLC with self-gravity: the flux-based versions call
    the solver with the old state (_self_gravity.py:286-312), whose switch
    reads that state's neighbours along every axis."""
    cfg, prm, rv, s = grav_case(2, 24, version=version, riemann=riemann)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 4
    assert rel_err(got, ref) < TOL


def test_compression_switch_split_3d_reflective(cuda):
    """The same in 3D with the split sweeps and reflective walls (both
    gravity face kernels, the boundary map with its sign flips); FP64 to the
    oracle, FP32 within 1e-5 relative L1 of it."""
    cfg, prm, rv, s = grav_case(3, 12, version=DONOR_ACCOUNTING, riemann=HYBRID_HLLC, boundary=REFLECTIVE_BOUNDARY,
                                split=True)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < TOL
    got32 = amx.time_integration(s.astype(np.float32), cfg, prm, rv)
    for row in range(got32.shape[0]):
        assert rel_l1(got32, ref, row=row) < 1e-5, row


@pytest.mark.parametrize("version", [RIEMANN_SPLIT, RIEMANN_SPLIT_UNSTABLE])
@pytest.mark.parametrize("riemann", [HLLC, HLLC_LM])
def test_riemann_split_versions_fp64(cuda, version, riemann):
    cfg, prm, rv, s = grav_case(2, 24, version=version, riemann=riemann)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < TOL


def test_open_boundaries_hockney_eastwood_fp64(cuda):
    cfg, prm, rv, s = grav_case(2, 24, version=RIEMANN_SPLIT, riemann=HLLC, boundary=OPEN_BOUNDARY)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < TOL


def test_split_3d_reflective_fp64(cuda):
    """The reference's collapse setting: split MUSCL-Hancock, HLLC,
    RIEMANN_SPLIT_UNSTABLE, reflective walls (open-boundary Poisson solve)."""
    cfg, prm, rv, s = grav_case(3, 12, version=RIEMANN_SPLIT_UNSTABLE, riemann=HLLC, boundary=REFLECTIVE_BOUNDARY,
                                split=True)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 10
    assert rel_err(got, ref) < TOL


@pytest.mark.parametrize("boundary", [PERIODIC_BOUNDARY, OPEN_BOUNDARY])
def test_1d_fp64(cuda, boundary):
    cfg, prm, rv, s = grav_case(1, 64, version=HALF_SPLIT, riemann=HLLC, boundary=boundary)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < TOL
    cfg, prm, rv, s = grav_case(1, 64, version=DONOR_ACCOUNTING, riemann=HLL, boundary=boundary, first_order=True)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < TOL


def test_split_2d_fp64(cuda):
    cfg, prm, rv, s = grav_case(2, 24, version=DONOR_ACCOUNTING, riemann=HLLC, split=True)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < TOL


@pytest.mark.parametrize("dim", [2, 3])
def test_mhd_fp64(cuda, dim):
    cfg, prm, rv, s = grav_case(dim, 24 if dim == 2 else 12, version=DONOR_ACCOUNTING, riemann=HLL, mhd=True)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 4
    assert rel_err(got, ref) < TOL


def test_periodic_roll_fp64(cuda):
    cfg, prm, rv, s = grav_case(2, 24, version=DONOR_ACCOUNTING, riemann=HLLC, roll=True)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert rel_err(got, ref) < TOL


def test_fp32_against_fp64_oracle(cuda):
    cfg, prm, rv, s = grav_case(2, 48, version=DONOR_ACCOUNTING, riemann=HLLC, dtype=np.float32, t_end=0.05)
    got, ref, _ = run_both(cfg, prm, rv, s)
    assert got.dtype == np.float32
    assert rel_l1(got, ref) < 1e-5


def test_gravity_changes_the_result(cuda):
    """The source term is not a no-op: the run differs from the run without gravity."""
    cfg, prm, rv, s = grav_case(2, 24)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    plain = amx.time_integration(s.copy(), cfg._replace(self_gravity=False), prm, rv)
    assert np.abs(got - plain).max() > 1e-4


def test_snapshot_gravitational_energy_fp64(cuda):
    from astronomix_gb300 import SnapshotSettings

    cfg, prm, rv, s = grav_case(2, 24, t_end=0.02)
    cfg = cfg._replace(return_snapshots=True, num_snapshots=3,
                       snapshot_settings=SnapshotSettings(return_states=True, return_total_energy=True,
                                                          return_gravitational_energy=True))
    snap = amx.time_integration(s.copy(), cfg, prm, rv)
    for i in range(3):
        st = snap.states[i]
        eg = ograv.gravitational_energy(st, cfg, rv, prm.gravitational_constant)
        assert abs(snap.gravitational_energy[i] - eg) <= 1e-12 * abs(eg)
        tot = odriver.snapshot_quantities(st, cfg, prm, rv).total_energy + eg
        assert abs(snap.total_energy[i] - tot) <= 1e-12 * abs(tot)


def test_abi_rejects_unsupported(cuda):
    cfg, prm, rv, s = grav_case(2, 16, version=RIEMANN_SPLIT, riemann=HLL)
    from astronomix_gb300.time_integration import make_amx_config

    c = make_amx_config(cfg, rv, s.shape, np.float64)
    with pytest.raises(_native.AmxError):
        _native.Plan(c)


@pytest.mark.parametrize("version", [RIEMANN_SPLIT_UNSTABLE, DONOR_ACCOUNTING, SIMPLE_SOURCE_TERM])
def test_evrard_collapse_fp64(cuda, version):
    """The reference's self-gravity problem (density contrast 1e4, reflective
    walls, open Poisson solve) at 16^3 for 12 steps."""
    from astronomix_gb300.initial_conditions import evrard_collapse

    cfg, prm, rv, s = evrard_collapse(16, dtype=np.float64, t_end=0.012, version=version)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] == 12
    assert rel_err(got, ref) < TOL


def test_evrard_collapse_energy_budget_fp32(cuda):
    """32^3 collapse to t = 0.3 in FP32: mass is conserved (reflective walls)
    and the gravitational energy turns into kinetic energy while the total
    (internal + kinetic + gravitational) drifts by less than 2 % of |E_grav|."""
    from astronomix_gb300 import SnapshotSettings
    from astronomix_gb300.initial_conditions import evrard_collapse

    cfg, prm, rv, s = evrard_collapse(32, dtype=np.float32, t_end=0.3)
    cfg = cfg._replace(return_snapshots=True, num_snapshots=4,
                       snapshot_settings=SnapshotSettings(return_total_mass=True, return_total_energy=True,
                                                          return_kinetic_energy=True,
                                                          return_gravitational_energy=True))
    snap = amx.time_integration(s.copy(), cfg, prm, rv)
    m = snap.total_mass
    assert abs(m[-1] - m[0]) < 1e-5 * m[0]
    eg, ek, et = snap.gravitational_energy, snap.kinetic_energy, snap.total_energy
    assert eg[0] < 0 and ek[0] < 1e-15  # (|u| carries the reference's 1e-20 under the root)
    assert ek[-1] > 1e-3 * abs(eg[0]) and eg[-1] < eg[0], (eg, ek)
    assert abs(et[-1] - et[0]) < 0.02 * abs(eg[0]), (et, eg, ek)


def test_split_mhd_fp64(cuda):
    """Self-gravity after both gas half-updates of the Pang-Wu split with the
    split MUSCL-Hancock scheme."""
    cfg, prm, rv, s = grav_case(2, 24, version=DONOR_ACCOUNTING, riemann=HLLC, mhd=True, split=True)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] >= 4
    assert rel_err(got, ref) < TOL


def test_fixed_timestep_fp64(cuda):
    cfg, prm, rv, s = grav_case(2, 24, version=HALF_SPLIT, riemann=HLL)
    cfg = cfg._replace(fixed_timestep=True, num_timesteps=7)
    got, ref, rec = run_both(cfg, prm, rv, s)
    assert rec["steps"] == 7
    assert rel_err(got, ref) < TOL


def test_step_seams_with_gravity_fp64(cuda):
    """amx_evolve_state and amx_fv_hydro_rk2 include the source term, as
    _evolve_state_fv and _evolve_gas_state_unsplit do."""
    import torch
    from astronomix_gb300.time_integration import get_plan
    from oracle import fv as ofv

    cfg, prm, rv, s = grav_case(2, 16, version=DONOR_ACCOUNTING, riemann=HLL, roll=True)
    plan = get_plan(cfg, rv, s.shape, np.float64)
    dev = torch.from_numpy(s.copy()).cuda()
    st = torch.cuda.current_stream().cuda_stream
    plan.reset(st)
    dt = 2e-3
    plan.evolve(dev.data_ptr(), _native.make_params(prm), dt, st)
    torch.cuda.synchronize()
    ref = ofv.evolve_state_fv(s.copy(), np.float64(dt), np.float64(prm.gamma), cfg, rv,
                              G=prm.gravitational_constant)
    assert rel_err(dev.cpu().numpy(), ref) < TOL
    # the gas-update seam: the RK2 update followed by the source term
    dev2 = torch.from_numpy(s.copy()).cuda()
    plan.hydro_rk2(dev2.data_ptr(), _native.make_params(prm), dt, st)
    torch.cuda.synchronize()
    ref2 = ofv.evolve_gas(s.copy(), np.float64(dt), np.float64(prm.gamma), cfg, rv, G=prm.gravitational_constant)
    assert rel_err(dev2.cpu().numpy(), ref2) < TOL
