"""Host side of the batched ensemble: the Gaussian-random-field initial
conditions (after astronomix/initial_condition_generation/
turbulent_ic_generator.py:19-109) and the checks that a batch shares one
configuration template.  No GPU needed."""

import numpy as np
import pytest

from astronomix_gb300 import HLL
from astronomix_gb300.ensemble import (create_turb_field, turbulent_ensemble_member, Ensemble, ENSEMBLE_SIZES)


def test_grf_is_real_zero_mean_and_seeded():
    a = create_turb_field(64, 1.0, -2.0, 1, 20, seed=3, dimensionality=2)
    b = create_turb_field(64, 1.0, -2.0, 1, 20, seed=3, dimensionality=2)
    c = create_turb_field(64, 1.0, -2.0, 1, 20, seed=4, dimensionality=2)
    assert a.shape == (64, 64) and a.dtype == np.float64
    assert np.array_equal(a, b)
    assert not np.allclose(a, c)
    assert abs(a.mean()) < 1e-12 * np.abs(a).max()
    f3 = create_turb_field(16, 1.0, -1.5, 1, 5, seed=0, dimensionality=3)
    assert f3.shape == (16, 16, 16) and abs(f3.mean()) < 1e-12


def test_grf_spectrum_slope_and_band():
    """Per-mode power of an amplitude slope of -2 falls as k^-4 inside the band
    and vanishes outside it (averaged over seeds)."""
    n, kmax = 128, 40
    k1 = np.fft.fftfreq(n) * n
    K = np.sqrt(np.add.outer(k1 ** 2, k1 ** 2))
    P = np.zeros((n, n))
    for seed in range(6):
        P += np.abs(np.fft.fftn(create_turb_field(n, 1.0, -2.0, 1, kmax, seed=seed, dimensionality=2))) ** 2
    assert P[K > kmax].max() < 1e-20 * P.max()
    assert P[0, 0] < 1e-20 * P.max()
    bins = np.arange(2, 30, 2)
    kc, pw = [], []
    for lo, hi in zip(bins[:-1], bins[1:]):
        m = (K >= lo) & (K < hi)
        kc.append(K[m].mean())
        pw.append(P[m].mean())
    slope = np.polyfit(np.log(kc), np.log(pw), 1)[0]
    assert -4.4 < slope < -3.6, slope


def test_ensemble_member_matches_its_recipe():
    for seed in range(6):
        cfg, prm, rv, s = turbulent_ensemble_member(seed)
        n = cfg.num_cells
        assert n in ENSEMBLE_SIZES
        assert s.shape == (7, n, n) and s.dtype == np.float32
        assert 0.05 <= prm.t_end <= 0.2
        assert prm.gamma == pytest.approx(5 / 3)
        assert np.all(s[0] == 1.0) and np.all(s[3] == 1.0)
        v_rms = np.sqrt(np.mean(s[1].astype(np.float64) ** 2 + s[2].astype(np.float64) ** 2))
        assert v_rms == pytest.approx(np.sqrt(5 / 3), rel=1e-5)  # rms Mach 1
        beta = 2 * 1.0 / s[4].astype(np.float64) ** 2
        assert np.allclose(beta, 1.0, rtol=1e-6)
        assert np.all(s[5] == 0) and np.all(s[6] == 0)
    # the draws are reproducible
    a = turbulent_ensemble_member(7)[3]
    b = turbulent_ensemble_member(7)[3]
    assert np.array_equal(a, b)


def test_batch_template_mismatch_is_rejected_on_the_host():
    ms = [turbulent_ensemble_member(s, size_override=16) for s in (0, 1)]
    shapes = [m[3].shape for m in ms]
    with pytest.raises(ValueError):
        Ensemble([ms[0][0], ms[1][0]._replace(riemann_solver=HLL)], [ms[0][1], ms[1][1]], ms[0][2], shapes)
    with pytest.raises(ValueError):
        Ensemble([ms[0][0], ms[1][0]], [ms[0][1], ms[1][1]._replace(gamma=1.4)], ms[0][2], shapes)
    with pytest.raises(ValueError):
        Ensemble([ms[0][0]], [ms[0][1], ms[1][1]], ms[0][2], shapes)
