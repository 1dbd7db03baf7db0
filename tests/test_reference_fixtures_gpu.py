"""The CUDA path against results of the reference's own code (tests/golden/reference_fixtures.npz).

Every run case of tests/golden/reference_cases.py, computed by leo1200/astronomix's
`time_integration` (on a NumPy stand-in for JAX, float64), is recomputed here by
the FP64 kernels through the C ABI: within 1e-12 relative to each field
group's scale, except the FD blast with a zero face-normal field, whose
eigenvector normalisation is ill-conditioned (a 1e-15 perturbation of the
input moves the reference's own result by ~1e-8), held to 1e-7.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import astronomix_gb300 as amx  # noqa: E402
import reference_cases as rc  # noqa: E402
from _cases import rel_err  # noqa: E402

pytestmark = pytest.mark.gpu

FIX = np.load(os.path.join(HERE, "golden", "reference_fixtures.npz"))
TOL = {"fd_blast12_zero_normal_field": 1e-7}


@pytest.mark.parametrize("name", sorted(rc.RUN_CASES))
def test_cuda_time_integration_matches_reference(cuda, name):
    cfg, prm, rv, s = rc.RUN_CASES[name]()
    got = amx.time_integration(np.array(s, dtype=np.float64), cfg, prm, rv)
    ref = FIX[name + "/output"]
    assert got.shape == ref.shape
    assert rel_err(got, ref) < TOL.get(name, 1e-12)


def test_cuda_fd_step_matches_reference(cuda):
    """One _evolve_state_fd step (dt 2e-3) of a random 3D MHD state with random face fields."""
    import torch
    from astronomix_gb300 import _native
    from astronomix_gb300.time_integration import get_plan
    from oracle import fd as ofd
    from _cases import blast_fd

    cfg, prm, rv, _ = blast_fd(n=8)
    U = rc.cons3d_mhd(13)
    bx, by, bz = rc.faces3d(13)
    P = np.concatenate([ofd.prim_from_cons(U, 1e-14, 1e-14, 5 / 3), np.stack([bx, by, bz])])
    plan = get_plan(cfg, rv, P.shape, np.float64)
    dev = torch.from_numpy(P.copy()).cuda()
    plan.evolve(dev.data_ptr(), _native.make_params(prm), 2e-3, torch.cuda.current_stream().cuda_stream)
    assert rel_err(dev.cpu().numpy(), FIX["evolve_state_fd/output"]) < 1e-12


def test_cuda_cfl_fd_matches_reference(cuda):
    import torch
    from astronomix_gb300 import _native
    from astronomix_gb300.time_integration import get_plan
    from oracle import fd as ofd
    from _cases import blast_fd

    cfg, prm, rv, _ = blast_fd(n=8)
    P = np.concatenate([ofd.prim_from_cons(rc.cons3d_mhd(7), 1e-14, 1e-14, 5 / 3), np.ones((3, 8, 8, 8))])
    plan = get_plan(cfg, rv, P.shape, np.float64)
    dev = torch.from_numpy(P).cuda()
    dt = plan.cfl_dt(dev.data_ptr(), _native.make_params(prm._replace(C_cfl=1.5, dt_max=1.0)),
                     torch.cuda.current_stream().cuda_stream)
    assert dt == pytest.approx(float(FIX["cfl_fd/output"]), rel=1e-14)
