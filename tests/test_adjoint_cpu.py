"""The oracle's reverse mode (torch.autograd through the NumPy/torch
restatement), which stands in for jax.grad of the reference in the adjoint
tests: with a fixed time step it matches central finite differences."""

import numpy as np
import pytest

from oracle import driver
from oracle._xp import backend

from _cases import smooth_random


@pytest.mark.parametrize("mhd", [False, True])
def test_oracle_autograd_matches_finite_differences(mhd):
    import torch

    cfg, prm, rv, s = smooth_random(2, 8, seed=2, mhd=mhd, t_end=0.006)
    cfg = cfg._replace(fixed_timestep=True, num_timesteps=3)
    rng = np.random.default_rng(0)
    w = torch.from_numpy(rng.standard_normal(s.shape))

    def loss(x):
        with backend("torch"):
            out = driver.time_integration(x, cfg, prm, rv, time_mode="float64")
        return (out * w).sum()

    x = torch.tensor(s, requires_grad=True)
    loss(x).backward()
    g = x.grad.numpy()
    eps = 1e-6
    for _ in range(2):
        d = rng.standard_normal(s.shape)
        with torch.no_grad():
            lp = float(loss(torch.from_numpy(s + eps * d)))
            lm = float(loss(torch.from_numpy(s - eps * d)))
        fd = (lp - lm) / (2 * eps)
        ad = float((g * d).sum())
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)
