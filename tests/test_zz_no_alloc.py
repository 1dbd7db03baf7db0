"""The allocation-free FV entry point, amx_fv_run_noalloc, against amx_run.

Callers that cannot allocate device memory -- a framework such as XLA that
owns the GPU's memory, a process held to a fixed memory budget, a loop that
cannot afford an allocation's implicit synchronisation -- use
amx_fv_run_noalloc, whose scratch lives in a fixed 8 MiB __device__ array
inside the library.  These tests call it through the C ABI and check that it
produces what the plan-based entry point produces, on two calls in a row
(the second call reuses the array the first one left behind), and that a
grid whose scratch does not fit is refused.

This file is collected last on purpose: a failure here leaves every other
test already run.
"""

import ctypes

import numpy as np
import pytest

from astronomix_gb300 import _native
from astronomix_gb300.time_integration import make_amx_config

from astronomix_gb300 import HLLC, HLLC_LM, SPLIT, MUSCL, VAN_ALBADA_PP
from _cases import orszag_tang, sod, smooth_random, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _case(case):
    """(cfg, prm, rv, state, steps) of each scratch layout the entry point lays out."""
    if case == "sod_fp64":
        cfg, prm, rv, s = sod(t_end=0.2)
        return cfg, prm, rv, s, 40
    if case == "sod_split_fp64":  # the split sweeps' third buffer shares the iterate region
        cfg, prm, rv, s = sod(riemann=HLLC, t_end=0.1)
        return cfg._replace(split=SPLIT, time_integrator=MUSCL), prm, rv, s, 30
    if case == "ot_split_fp64":
        cfg, prm, rv, s = orszag_tang(n=48, t_end=0.02, riemann=HLLC)
        return cfg._replace(split=SPLIT, time_integrator=MUSCL), prm, rv, s, 10
    if case == "hydro3d_hllc_lm_fp64":
        cfg, prm, rv, s = smooth_random(3, 16, seed=4, riemann=HLLC_LM, t_end=0.02)
        return cfg, prm, rv, s, 8
    if case == "mhd3d_fp32":
        cfg, prm, rv, s = smooth_random(3, 16, seed=5, mhd=True, dtype=np.float32, t_end=0.02)
        return cfg, prm, rv, s.astype(np.float32), 6
    if case == "mhd2d_van_albada_pp_fp64":
        cfg, prm, rv, s = smooth_random(2, 32, seed=6, mhd=True, limiter=VAN_ALBADA_PP, t_end=0.02)
        return cfg, prm, rv, s, 8
    dtype = np.float64 if case == "ot_fp64" else np.float32
    cfg, prm, rv, s = orszag_tang(n=64, t_end=0.02, dtype=dtype)
    return cfg, prm, rv, s, 12


def _noalloc(lib, cfg_c, state, prm_c, steps, stream):
    info = _native.amx_run_info()
    rc = lib.amx_fv_run_noalloc(ctypes.byref(cfg_c), ctypes.c_void_p(state.data_ptr()), ctypes.byref(prm_c),
                                int(steps), ctypes.byref(info), ctypes.c_void_p(stream))
    return rc, info


@pytest.mark.parametrize("case", ["ot_fp64", "ot_fp32", "sod_fp64", "sod_split_fp64", "ot_split_fp64",
                                  "hydro3d_hllc_lm_fp64", "mhd3d_fp32", "mhd2d_van_albada_pp_fp64"])
def test_noalloc_matches_plan_entry_point_twice(cuda, case):
    import torch

    lib = _native.lib()
    cfg, prm, rv, s, steps = _case(case)
    cfg_c = make_amx_config(cfg, rv, s.shape, s.dtype)
    prm_c = _native.make_params(prm)
    stream = torch.cuda.current_stream().cuda_stream

    # existing entry point: a plan with its own workspace
    plan = _native.Plan(make_amx_config(cfg, rv, s.shape, s.dtype))
    ref = torch.from_numpy(s.copy()).cuda()
    ref_info = plan.run(ref.data_ptr(), prm_c, steps, stream)
    ref_np = ref.cpu().numpy()

    for call in range(2):
        got = torch.from_numpy(s.copy()).cuda()
        rc, info = _noalloc(lib, cfg_c, got, prm_c, steps, stream)
        assert rc == 0, "call %d returned %d" % (call, rc)
        torch.cuda.synchronize()
        assert info.steps == ref_info.steps, (call, info.steps, ref_info.steps)
        assert info.t == pytest.approx(ref_info.t, rel=1e-12)
        assert info.status == 0
        if s.dtype == np.float32:
            # the same kernel on the same grid: bit for bit
            assert np.array_equal(got.cpu().numpy(), ref_np), call
        else:
            assert rel_err(got.cpu().numpy(), ref_np) < FP64_TOL, call


def test_noalloc_refuses_grids_beyond_its_scratch(cuda):
    import torch

    lib = _native.lib()
    cfg, prm, rv, s = orszag_tang(n=512, t_end=0.01, dtype=np.float64)
    cfg_c = make_amx_config(cfg, rv, s.shape, s.dtype)
    prm_c = _native.make_params(prm)
    state = torch.from_numpy(s.copy()).cuda()
    before = state.clone()
    rc, _ = _noalloc(lib, cfg_c, state, prm_c, 1, torch.cuda.current_stream().cuda_stream)
    assert rc == _native.AMX_ERR_TOO_LARGE
    torch.cuda.synchronize()
    assert torch.equal(state, before)


def test_noalloc_refuses_what_needs_allocation(cuda):
    """FD, self-gravity and turbulent forcing need workspace between the
    kernel's phases: refused before any launch."""
    import torch
    from _cases import blast_fd

    lib = _native.lib()
    stream = torch.cuda.current_stream().cuda_stream
    cfg, prm, rv, s = blast_fd(n=8)
    state = torch.from_numpy(s.copy()).cuda()
    rc, _ = _noalloc(lib, make_amx_config(cfg, rv, s.shape, s.dtype), state, _native.make_params(prm), 1, stream)
    assert rc == _native.AMX_ERR_UNSUPPORTED
    cfg, prm, rv, s = orszag_tang(n=32)
    c = make_amx_config(cfg, rv, s.shape, s.dtype)
    c.self_gravity = 1
    state = torch.from_numpy(s.copy()).cuda()
    rc, _ = _noalloc(lib, c, state, _native.make_params(prm), 1, stream)
    assert rc == _native.AMX_ERR_UNSUPPORTED


def test_noalloc_refuses_huge_grids_without_overflow(cuda):
    """A 3D grid whose cell count overflows 64 bits is refused as too large."""
    import torch

    lib = _native.lib()
    cfg, prm, rv, s = smooth_random(3, 8, seed=1, mhd=True)
    c = make_amx_config(cfg, rv, s.shape, s.dtype)
    c.num_cells = 1 << 22
    state = torch.from_numpy(s.copy()).cuda()
    rc, _ = _noalloc(lib, c, state, _native.make_params(prm), 1, torch.cuda.current_stream().cuda_stream)
    assert rc == _native.AMX_ERR_TOO_LARGE
