"""The oracle's compiled restatement of the FD step (oracle/cpu/fd_step.cpp)
against the NumPy oracle and against the reference's own results.

The restatement is the CPU baseline that bench.py times; these checks make
it a faithful one: FP64 runs equal the NumPy oracle bit for bit (the same
order of operations, no contraction), and the reference's own
time_integration results (tests/golden/reference_fixtures.npz) to 1e-12.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import reference_cases as rc  # noqa: E402
from oracle import cpu, driver  # noqa: E402
from _cases import blast_fd, rel_err, rel_l1  # noqa: E402

FIX = np.load(os.path.join(HERE, "golden", "reference_fixtures.npz"))


@pytest.mark.parametrize("name", ["fd_blast12_oblique", "fd_blast12_floors", "fd_blast12_zero_normal_field"])
def test_restatement_matches_reference_and_oracle(name):
    cfg, prm, rv, s = rc.RUN_CASES[name]()
    x = np.ascontiguousarray(np.array(s, dtype=np.float64))
    t, steps = cpu.fd_run(x, cfg, prm)
    assert t == pytest.approx(prm.t_end, abs=1e-15)
    assert rel_err(x, FIX[name + "/output"]) < 1e-12
    ref = driver.time_integration(np.array(s, dtype=np.float64), cfg, prm, rv)
    assert np.array_equal(x, ref)


def test_restatement_fp32_close_to_fp64():
    cfg, prm, rv, s = blast_fd(n=12, t_end=0.003, dtype=np.float32)
    x32 = np.ascontiguousarray(s.astype(np.float32))
    x64 = np.ascontiguousarray(s.astype(np.float64))
    cpu.fd_run(x32, cfg, prm)
    cpu.fd_run(x64, cfg, prm)
    assert rel_l1(x32, x64) < 1e-5


def test_restatement_threads_do_not_change_results():
    cfg, prm, rv, s = blast_fd(n=12, t_end=0.002, B=(0.6, 0.5, 0.4))
    a = np.ascontiguousarray(s.copy())
    b = np.ascontiguousarray(s.copy())
    cpu.fd_run(a, cfg, prm, nthreads=1)
    cpu.fd_run(b, cfg, prm, nthreads=4)
    assert np.array_equal(a, b)
