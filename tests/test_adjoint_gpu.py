"""Discrete adjoint of the FV time integration, through the C ABI.

FP64: the gradient of a random linear functional of the final state with
respect to the whole initial state equals torch.autograd through the oracle
(the stand-in for jax.grad of the reference: dt detached, the fixed point
differentiated through its iterations) to 1e-9, and central finite
differences of the replayed program (fixed schedule) to 1e-6.  The result
does not depend on the checkpoint interval.  FP32 gradients agree with FP64
ones to the stated tolerance.
"""

import numpy as np
import pytest

from astronomix_gb300.adjoint import AdjointIntegrator, time_integration_differentiable
from oracle import driver as odriver
from oracle._xp import backend

from _cases import smooth_random

pytestmark = pytest.mark.gpu


def oracle_grad(cfg, prm, rv, s, w):
    import torch

    x = torch.tensor(s, dtype=torch.float64, requires_grad=True)
    rec = {}
    with backend("torch"):
        out = odriver.time_integration(x, cfg, prm, rv, time_mode="float64", record=rec)
    (out * torch.from_numpy(w)).sum().backward()
    return x.grad.numpy(), out.detach().numpy(), rec


def gpu_grad(cfg, prm, rv, s, w, every=20, dtype=np.float64, tape_budget=0):
    import torch

    integ = AdjointIntegrator(cfg, prm, rv, s.shape, dtype, checkpoint_every=every, tape_budget=tape_budget)
    x = torch.from_numpy(s.astype(dtype)).cuda()
    y = integ.forward(x)
    g = integ.backward(torch.from_numpy(w.astype(dtype)).cuda())
    return g.cpu().numpy(), y.cpu().numpy(), integ


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


CASES = [
    ("2d_mhd", dict(dim=2, n=12, mhd=True, t_end=0.04)),
    ("2d_hydro", dict(dim=2, n=16, mhd=False, t_end=0.04)),
    ("3d_mhd", dict(dim=3, n=8, mhd=True, t_end=0.03)),
]


@pytest.mark.parametrize("tape", ["checkpoints", "stored"])
@pytest.mark.parametrize("name,kw", CASES, ids=[c[0] for c in CASES])
def test_fp64_gradient_matches_autograd_of_oracle(cuda, name, kw, tape):
    cfg, prm, rv, s = smooth_random(kw["dim"], kw["n"], seed=3, mhd=kw["mhd"], t_end=kw["t_end"])
    w = np.random.default_rng(7).standard_normal(s.shape)
    g_ref, y_ref, rec = oracle_grad(cfg, prm, rv, s, w)
    g, y, integ = gpu_grad(cfg, prm, rv, s, w, every=2, tape_budget=0 if tape == "checkpoints" else 1 << 30)
    assert integ.stored_tape() == (tape == "stored")
    dts, its = integ.schedule()
    assert len(dts) == rec["steps"] >= 3
    if kw["mhd"]:
        assert its == rec["magnetic_iterations"]
    assert rel(y, y_ref) < 1e-12
    assert rel(g, g_ref) < 1e-9, rel(g, g_ref)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_checkpoint_interval_and_stored_tape_give_the_same_gradient(cuda, dtype):
    """Checkpoint intervals 1, 3, 50, the whole tape stored by the forward
    kernel, and a tape budget too small for the run (which falls back to
    checkpoints) all give the same gradient and the same final state."""
    cfg, prm, rv, s = smooth_random(2, 12, seed=4, mhd=True, t_end=0.04)
    if dtype == np.float32:
        cfg = cfg._replace(numerical_precision=0)
    s = s.astype(dtype)
    w = np.random.default_rng(1).standard_normal(s.shape)
    runs = [gpu_grad(cfg, prm, rv, s, w, every=e, dtype=dtype) for e in (1, 3, 50)]
    stored = gpu_grad(cfg, prm, rv, s, w, dtype=dtype, tape_budget=1 << 28)
    small = gpu_grad(cfg, prm, rv, s, w, every=4, dtype=dtype, tape_budget=s.nbytes * 6)
    assert stored[2].stored_tape() and not small[2].stored_tape()
    for g, y, _ in runs[1:] + [stored, small]:
        assert np.array_equal(g, runs[0][0])
        assert np.array_equal(y, runs[0][1])


def test_fp64_gradient_matches_finite_differences_of_replay(cuda):
    import torch

    cfg, prm, rv, s = smooth_random(3, 8, seed=5, mhd=True, t_end=0.03)
    rng = np.random.default_rng(2)
    w = rng.standard_normal(s.shape)
    g, _, integ = gpu_grad(cfg, prm, rv, s, w)
    W = torch.from_numpy(w).cuda()
    eps = 1e-6
    for _ in range(3):
        d = rng.standard_normal(s.shape)
        xp = torch.from_numpy(s + eps * d).cuda()
        xm = torch.from_numpy(s - eps * d).cuda()
        lp = float((integ.replay(xp) * W).sum())
        lm = float((integ.replay(xm) * W).sum())
        fd = (lp - lm) / (2 * eps)
        ad = float((g * d).sum())
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_fp32_gradient_close_to_fp64(cuda):
    cfg, prm, rv, s = smooth_random(2, 24, seed=6, mhd=True, t_end=0.04)
    w = np.random.default_rng(3).standard_normal(s.shape)
    g64, _, _ = gpu_grad(cfg, prm, rv, s, w, dtype=np.float64)
    cfg32 = cfg._replace(numerical_precision=0)
    g32, _, _ = gpu_grad(cfg32, prm, rv, s.astype(np.float32), w, dtype=np.float32)
    err = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
    assert err < 1e-4, err


def test_autograd_function_backward(cuda):
    import torch

    cfg, prm, rv, s = smooth_random(2, 12, seed=8, mhd=True, t_end=0.04)
    x = torch.from_numpy(s).cuda().requires_grad_(True)
    y = time_integration_differentiable(x, cfg, prm, rv, checkpoint_every=4)
    target = torch.ones_like(y[0])
    loss = ((y[0].double() - target) ** 2).mean()
    loss.backward()
    w = np.zeros(s.shape)
    w[0] = 2 * (y[0].detach().cpu().numpy() - 1.0) / y[0].numel()
    g_ref, _, _ = oracle_grad(cfg, prm, rv, s, w)
    assert rel(x.grad.cpu().numpy(), g_ref) < 1e-9
