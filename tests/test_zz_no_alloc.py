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

from _cases import orszag_tang, sod, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _noalloc(lib, cfg_c, state, prm_c, steps, stream):
    info = _native.amx_run_info()
    rc = lib.amx_fv_run_noalloc(ctypes.byref(cfg_c), ctypes.c_void_p(state.data_ptr()), ctypes.byref(prm_c),
                                int(steps), ctypes.byref(info), ctypes.c_void_p(stream))
    return rc, info


@pytest.mark.parametrize("case", ["ot_fp64", "ot_fp32", "sod_fp64"])
def test_noalloc_matches_plan_entry_point_twice(cuda, case):
    import torch

    lib = _native.lib()
    if case == "sod_fp64":
        cfg, prm, rv, s = sod(t_end=0.2)
        steps = 40
    else:
        dtype = np.float64 if case == "ot_fp64" else np.float32
        cfg, prm, rv, s = orszag_tang(n=64, t_end=0.02, dtype=dtype)
        steps = 12
    cfg_c = make_amx_config(cfg, rv, s.shape, s.dtype)
    prm_c = _native.make_params(prm)
    stream = torch.cuda.current_stream().cuda_stream

    # existing entry point: a plan with its own workspace
    plan = _native.Plan(make_amx_config(cfg, rv, s.shape, s.dtype))
    ref = torch.from_numpy(s.copy()).cuda()
    ref_info = plan.run(ref.data_ptr(), prm_c, steps, stream)
    ref_np = ref.cpu().numpy()
    tol = FP64_TOL if s.dtype == np.float64 else 1e-6

    for call in range(2):
        got = torch.from_numpy(s.copy()).cuda()
        rc, info = _noalloc(lib, cfg_c, got, prm_c, steps, stream)
        assert rc == 0, "call %d returned %d" % (call, rc)
        torch.cuda.synchronize()
        assert info.steps == ref_info.steps, (call, info.steps, ref_info.steps)
        assert info.t == pytest.approx(ref_info.t, rel=1e-12)
        assert info.status == 0
        assert rel_err(got.cpu().numpy(), ref_np) < tol, call


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
