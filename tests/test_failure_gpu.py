"""Failure detection of the CUDA path, provoked from the host (no GPU fault).

The reference's numerical failures are silent unless `runtime_debugging` is
set, which wraps the run in checkify (time_integration.py:142-161): then a
NaN, or a magnetic fixed point that stopped at its 1000-iteration cap
(_magnetic_field_update.py:127-141, checked at :176-206), raises.  Here the
kernels record status bits (never a trap), the host raises
FloatingPointError for them under runtime_debugging and returns the
state otherwise.  The grid barrier of the persistent kernel gives up after a
bounded number of polls; a test sets that bound to one poll so that the wait
runs out, and the kernel returns AMX_ERR_TIMEOUT with every block exited.
"""

import numpy as np
import pytest

import astronomix_gb300 as amx
from astronomix_gb300 import _native
from astronomix_gb300.time_integration import make_amx_config, _raise_status
from oracle import driver as odriver
from oracle import fv as ofv

from _cases import orszag_tang, blast_fd, smooth_random, rel_err

pytestmark = pytest.mark.gpu


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def test_nan_input_fv_raises_under_runtime_debugging(cuda):
    cfg, prm, rv, s = orszag_tang(n=32, t_end=0.01)
    s = s.copy()
    s[0, 5, 7] = np.nan
    with pytest.raises(FloatingPointError):
        amx.time_integration(s.copy(), cfg._replace(runtime_debugging=True), prm, rv)
    out = amx.time_integration(s.copy(), cfg, prm, rv)  # silent, like the reference
    assert np.isnan(out).any()


def test_nan_input_fd_raises_under_runtime_debugging(cuda):
    cfg, prm, rv, s = blast_fd(n=16, t_end=0.003)
    s = s.copy()
    s[4, 3, 4, 5] = np.nan
    with pytest.raises(FloatingPointError):
        amx.time_integration(s.copy(), cfg._replace(runtime_debugging=True), prm, rv)
    out = amx.time_integration(s.copy(), cfg, prm, rv)
    assert np.isnan(out).any()


def test_fixed_point_cap_sets_not_converged_and_matches_capped_oracle(cuda, monkeypatch):
    """With the cap at 2 iterations the update stops early exactly where the
    oracle with the same cap stops, and the status says so."""
    import torch

    cfg, prm, rv, s = smooth_random(2, 16, seed=3, mhd=True, t_end=0.02)
    plan = _native.Plan(make_amx_config(cfg, rv, s.shape, np.float64))
    plan.set_limits(2, 0)
    dev = torch.from_numpy(s.copy()).cuda()
    plan.reset(_stream())
    info = plan.run(dev.data_ptr(), _native.make_params(prm), 1 << 40, _stream())
    assert info.status & _native.AMX_ERR_NOT_CONVERGED
    assert not info.status & ~_native.AMX_ERR_NOT_CONVERGED
    with pytest.raises(FloatingPointError):
        _raise_status(info.status, cfg._replace(runtime_debugging=True))
    _raise_status(info.status, cfg)  # silent without runtime_debugging
    monkeypatch.setattr(ofv, "MAX_FIXED_POINT_ITERATIONS", 2)
    ref = odriver.time_integration(s.copy(), cfg, prm, rv)
    assert rel_err(dev.cpu().numpy(), ref) < 1e-12
    # back to the reference's cap: converged, no status
    plan.set_limits(0, 0)
    dev = torch.from_numpy(s.copy()).cuda()
    plan.reset(_stream())
    info = plan.run(dev.data_ptr(), _native.make_params(prm), 1 << 40, _stream())
    assert info.status == 0


def test_barrier_timeout_returns_status_and_plan_recovers(cuda):
    """A one-poll barrier limit makes the first barrier's wait run out: the
    launch returns with AMX_ERR_TIMEOUT (raised as AmxError), and the same
    plan then runs normally once the limit is restored."""
    import torch

    cfg, prm, rv, s = smooth_random(3, 32, seed=4, mhd=True, t_end=0.01)
    plan = _native.Plan(make_amx_config(cfg, rv, s.shape, np.float64))
    plan.set_limits(0, 1)
    dev = torch.from_numpy(s.copy()).cuda()
    plan.reset(_stream())
    info = plan.run(dev.data_ptr(), _native.make_params(prm), 1 << 40, _stream())
    assert info.status & _native.AMX_ERR_TIMEOUT
    with pytest.raises(_native.AmxError):
        _raise_status(info.status, cfg)
    plan.set_limits(0, 0)
    dev = torch.from_numpy(s.copy()).cuda()
    plan.reset(_stream())
    info = plan.run(dev.data_ptr(), _native.make_params(prm), 1 << 40, _stream())
    assert info.status == 0
    ref = odriver.time_integration(s.copy(), cfg, prm, rv)
    assert rel_err(dev.cpu().numpy(), ref) < 1e-12


def test_set_limits_rejects_fd_and_negative_values(cuda):
    cfg, prm, rv, s = blast_fd(n=16)
    fd_plan = _native.Plan(make_amx_config(cfg, rv, s.shape, np.float64))
    with pytest.raises(_native.AmxError):
        fd_plan.set_limits(5, 0)
    cfg, prm, rv, s = orszag_tang(n=16)
    plan = _native.Plan(make_amx_config(cfg, rv, s.shape, np.float64))
    with pytest.raises(_native.AmxError):
        plan.set_limits(-1, 0)
