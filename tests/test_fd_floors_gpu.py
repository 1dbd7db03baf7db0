"""FD WENO-CT with its positivity floors active, and the FD diagnostics, vs the oracle.

The floors act in three places of the reference: `_enforce_positivity` before
every stage but the last and after the step
(_finite_difference/_fluid_equations/_enforce_positivity.py:24-59,
_ssprk.py:285-292, :340-347), the primitive conversion inside the flux
(_equations.py:140-150) and the eigensystem's building blocks, where each
`jnp.where` re-tests its condition on the values already floored
(_eigen.py:61-74, :140-150).  The blast below sits under both floors: its
ambient pressure 0.1 is below minimum_pressure 0.2, and a low-density blob
(rho = 0.3) is below minimum_density 0.5.
"""

import numpy as np
import pytest

import astronomix_gb300 as amx
from astronomix_gb300 import _native
from astronomix_gb300.time_integration import get_plan
from oracle import driver as odriver
from oracle import fd as ofd

from _cases import blast_fd, rel_err, rel_l1

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def floored_blast(n=16, dtype=np.float64, t_end=0.003):
    cfg, prm, rv, s = blast_fd(n=n, t_end=t_end, B=(0.6, 0.5, 0.4), rhomin=0.5, pmin=0.2)
    x = (np.arange(n) + 0.5) / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    blob = (X - 0.25) ** 2 + (Y - 0.3) ** 2 + (Z - 0.7) ** 2 < 0.15 ** 2
    s = s.copy()
    s[0] = np.where(blob, 0.3, s[0])
    return cfg, prm, rv, s.astype(dtype)


def test_floors_are_active_in_the_initial_state():
    cfg, prm, rv, s = floored_blast()
    assert (s[0] < prm.minimum_density).sum() > 0
    assert (s[4] < prm.minimum_pressure).sum() > 0.5 * s[4].size


def test_fd_floors_single_step_fp64(cuda):
    import torch

    cfg, prm, rv, s = floored_blast()
    plan = get_plan(cfg, rv, s.shape, np.float64)
    dev = torch.from_numpy(s.copy()).cuda()
    dt = 1e-3
    plan.evolve(dev.data_ptr(), _native.make_params(prm), dt, torch.cuda.current_stream().cuda_stream)
    got = dev.cpu().numpy()
    ref = ofd.evolve_state_fd(s.copy(), dt, prm.gamma, cfg.grid_spacing, prm.minimum_density,
                              prm.minimum_pressure)
    assert rel_err(got, ref) < FP64_TOL
    # the floors shaped the result: the oracle without them differs
    free = ofd.evolve_state_fd(s.copy(), dt, prm.gamma, cfg.grid_spacing, 1e-14, 1e-14)
    assert rel_err(free, ref) > 1e-3


def test_fd_floors_cfl_fp64(cuda):
    import torch

    cfg, prm, rv, s = floored_blast()
    plan = get_plan(cfg, rv, s.shape, np.float64)
    dev = torch.from_numpy(s).cuda()
    dt = plan.cfl_dt(dev.data_ptr(), _native.make_params(prm), torch.cuda.current_stream().cuda_stream)
    ref = ofd.cfl_time_step_fd(s, cfg.grid_spacing, prm.dt_max, prm.gamma, prm.C_cfl, prm.minimum_density,
                               prm.minimum_pressure)
    assert dt == pytest.approx(float(ref), rel=1e-14)


def test_fd_floors_run_fp64(cuda):
    cfg, prm, rv, s = floored_blast()
    rec = {}
    ref = odriver.time_integration(s.copy(), cfg, prm, rv, record=rec)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    assert rec["steps"] >= 2
    assert rel_err(got, ref) < FP64_TOL
    assert got[0].min() >= prm.minimum_density and got[4].min() >= prm.minimum_pressure


def test_fd_floors_run_fp32_l1(cuda):
    cfg, prm, rv, s = floored_blast(dtype=np.float32)
    got = amx.time_integration(s.copy(), cfg, prm, rv)
    ref64 = odriver.time_integration(s.astype(np.float64), cfg, prm, rv)
    assert got.dtype == np.float32
    assert rel_l1(got, ref64) < 1e-5


def test_fd_divergence_diagnostic_fp64(cuda):
    """max |div B| of the face fields (_interface_field_divergence,
    _finite_difference/_maths/_differencing.py:33-51), as the snapshot
    diagnostic reports it (time_integration.py:507-522), on face fields
    with a divergence of order one."""
    import torch

    cfg, prm, rv, s = blast_fd(n=16)
    rng = np.random.default_rng(5)
    s = s.copy()
    s[8:11] += 0.1 * rng.standard_normal(s[8:11].shape)
    plan = get_plan(cfg, rv, s.shape, np.float64)
    dev = torch.from_numpy(s).cuda()
    sums = plan.conservation_sums(dev.data_ptr(), _native.make_params(prm), torch.cuda.current_stream().cuda_stream)
    ref = np.abs(ofd.interface_field_divergence(s[8], s[9], s[10], cfg.grid_spacing)).max()
    assert ref > 1.0
    assert sums[4] == pytest.approx(float(ref), rel=1e-12)
    snap = odriver.snapshot_quantities(s, cfg, prm, rv)
    assert sums[0] == pytest.approx(snap.total_mass, rel=1e-13)
    assert sums[1] == pytest.approx(snap.total_energy, rel=1e-12)
