"""Batched ensemble (one persistent launch for many 2D FV runs) through the C ABI.

A run's result must not depend on the batch it is in: every run of a batch
equals, bit for bit, the single-run path on the same input (which is itself
held to the oracle by the FV parity tests), in FP32 and FP64, whatever the
tile shape, resident-block count, graph replay or pause/resume.  One FP64
batch is also compared with the oracle directly (1e-12).
"""

import numpy as np
import pytest

import astronomix_gb300 as amx
from astronomix_gb300 import HLL
from astronomix_gb300.ensemble import Ensemble, time_integration_batched, turbulent_ensemble_member
from oracle import driver as odriver

from _cases import smooth_random, rel_err

pytestmark = pytest.mark.gpu

SIZES = (16, 24, 40, 32, 20)


def members(dtype, sizes=SIZES, t_scale=0.25):
    out = []
    for seed, n in enumerate(sizes):
        cfg, prm, rv, s = turbulent_ensemble_member(seed, dtype=dtype, size_override=n)
        prm = prm._replace(t_end=prm.t_end * t_scale)
        out.append((cfg, prm, rv, s))
    return out


def single_runs(ms):
    return [amx.time_integration(s.copy(), cfg, prm, rv) for cfg, prm, rv, s in ms]


def batched(ms, **kw):
    return time_integration_batched([m[3].copy() for m in ms], [m[0] for m in ms], [m[1] for m in ms], ms[0][2],
                                    **kw)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_batch_equals_single_runs_bitwise(cuda, dtype):
    ms = members(dtype)
    got, infos = batched(ms, return_info=True)
    ref = single_runs(ms)
    for i, (g, r) in enumerate(zip(got, ref)):
        assert g.dtype == dtype
        assert np.array_equal(g, r), (i, np.abs(g.astype(np.float64) - r).max())
    for info, m in zip(infos, ms):
        assert abs(info.t - m[1].t_end) <= 1e-12  # exact end time
        assert info.steps > 0
        assert info.status == 0


def test_batch_fp64_matches_oracle(cuda):
    ms = members(np.float64, sizes=(16, 24), t_scale=0.1)
    got = batched(ms)
    for g, (cfg, prm, rv, s) in zip(got, ms):
        ref = odriver.time_integration(s.copy(), cfg, prm, rv)
        assert rel_err(g, ref) < 1e-12


def test_batch_hydro_hll(cuda):
    ms = []
    for seed, n in enumerate((16, 28, 20)):
        cfg, prm, rv, s = smooth_random(2, n, seed=seed, riemann=HLL, t_end=0.02 + 0.01 * seed)
        ms.append((cfg, prm, rv, s))
    got = batched(ms)
    for g, r in zip(got, single_runs(ms)):
        assert np.array_equal(g, r)


def _device(ms):
    import torch

    return [torch.from_numpy(m[3].copy()).cuda() for m in ms]


def test_tilings_graph_and_resume_identical(cuda):
    import torch

    ms = members(np.float32)
    shapes = [m[3].shape for m in ms]
    ens = Ensemble([m[0] for m in ms], [m[1] for m in ms], ms[0][2], shapes, np.float32)
    ref = single_runs(ms)
    tried = 0
    for variant in range(3):
        for bps in (1, 2):
            try:
                ens.batch.set_tiling(variant, bps)
            except amx._native.AmxError:
                continue
            tried += 1
            for use_graph in (False, True):
                ens.reset()
                st = _device(ms)
                ens.run(st, use_graph=use_graph)
                torch.cuda.synchronize()
                for i, (a, r) in enumerate(zip(st, ref)):
                    assert np.array_equal(a.cpu().numpy(), r), (variant, bps, use_graph, i)
    assert tried >= 4
    # pause after 5 lock-step steps, then finish (graph replays the same launch)
    ens.batch.set_tiling(0, 0)
    ens.reset()
    st = _device(ms)
    ens.run(st, max_steps=5)
    infos, lock = ens.info()
    assert lock == 5
    assert max(i.steps for i in infos) == 5
    ens.run(st)
    infos, lock = ens.info()
    assert lock == max(i.steps for i in infos)
    for a, r in zip(st, ref):
        assert np.array_equal(a.cpu().numpy(), r)


def test_tune_keeps_states_and_counters(cuda):
    import torch

    ms = members(np.float32, sizes=(24, 32, 16))
    shapes = [m[3].shape for m in ms]
    ens = Ensemble([m[0] for m in ms], [m[1] for m in ms], ms[0][2], shapes, np.float32)
    st = _device(ms)
    before = [a.clone() for a in st]
    res = ens.tune(st, steps=2)
    assert res["trial_ms"] > 0
    assert res["blocks_per_sm"] >= 1
    for a, b in zip(st, before):
        assert torch.equal(a, b)
    infos, lock = ens.info()
    assert lock == 0 and all(i.steps == 0 for i in infos)
    ens.run(st)
    torch.cuda.synchronize()
    for a, r in zip(st, single_runs(ms)):
        assert np.array_equal(a.cpu().numpy(), r)

