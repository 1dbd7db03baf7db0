"""CPU checks of the oracle itself: known answers, conservation, convergence, golden data.

The oracle is the checker of the CUDA kernels, so it is pinned first:
* the Sod shock tube against the exact Riemann solution (the reference uses
  ExactPack for this, tests/hydro_tests/shock_tube.py:109-134);
* second-order convergence on Gaussian-pulse advection
  (tests/hydro_tests/convergence.py:28-119);
* exact periodic conservation of mass, momentum and energy (FV) and
  round-off-level interface divergence of B (FD,
  tests/finite_difference/mhd_blast3D.py:253-279);
* the golden Orszag-Tang state shipped with the reference
  (tests/mhd_tests/final_state_orszag_tang.npz), through a committed summary.
"""

import json
import os

import numpy as np
import pytest

from astronomix_gb300 import (
    SimulationConfig, SimulationParams, BoundarySettings1D, finalize_config, get_registered_variables,
    construct_primitive_state, HLLC, DOUBLE_MINMOD, MINMOD, PERIODIC_BOUNDARY,
)
from oracle import driver, fv, fd, sod_exact

from _cases import sod, smooth_random, orszag_tang, blast_fd

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_sod_oracle_vs_exact_solution():
    cfg, prm, rv, s = sod(n=400, t_end=0.2)
    out = driver.time_integration(s, cfg, prm, rv)
    x = (np.arange(400) + 0.5) / 400
    rho, u, p = sod_exact.sample(x, 0.2, 0.5, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1), 1.4)
    dx = 1 / 400
    assert np.abs(out[0] - rho).sum() * dx < 3e-3
    assert np.abs(out[1] - u).sum() * dx < 6e-3
    assert np.abs(out[2] - p).sum() * dx < 3e-3


def test_exact_riemann_star_state_textbook_value():
    # Sod: p* = 0.30313, u* = 0.92745 (Toro, Table 4.2)
    p, u = sod_exact.star_state(1.0, 0.0, 1.0, 0.125, 0.0, 0.1, 1.4)
    assert p == pytest.approx(0.30313, abs=2e-5)
    assert u == pytest.approx(0.92745, abs=2e-5)


def _pulse_l1(n):
    cfg = SimulationConfig(dimensionality=1, box_size=1.0, num_cells=n, riemann_solver=HLLC, limiter=DOUBLE_MINMOD,
                           boundary_settings=BoundarySettings1D(PERIODIC_BOUNDARY, PERIODIC_BOUNDARY))
    rv = get_registered_variables(cfg)
    x = (np.arange(n) + 0.5) / n

    def exact(t):
        c = (0.5 + t) % 1.0
        d = np.abs(x - c)
        return 1.0 + np.exp(-d ** 2 / (2 * 0.0625 ** 2))

    s = construct_primitive_state(cfg, rv, density=exact(0.0), velocity_x=np.ones(n), gas_pressure=np.full(n, 10.0))
    cfg = finalize_config(cfg, s.shape)
    prm = SimulationParams(t_end=0.25, gamma=1.4, C_cfl=0.1)
    out = driver.time_integration(s, cfg, prm, rv)
    return np.abs(out[0] - exact(0.25)).sum() / n


def test_pulse_advection_second_order():
    e = [_pulse_l1(n) for n in (64, 128, 256)]
    rates = np.log2(np.array(e[:-1]) / np.array(e[1:]))
    assert np.all(rates > 1.6), (e, rates)


@pytest.mark.parametrize("dim", [2, 3])
def test_fv_periodic_conservation(dim):
    cfg, prm, rv, s = smooth_random(dim, 16 if dim == 2 else 8, seed=5, t_end=0.02)
    out = driver.time_integration(s, cfg, prm, rv)
    U0 = fv.conserved_state_from_primitive(s, prm.gamma, dim, rv)
    U1 = fv.conserved_state_from_primitive(out, prm.gamma, dim, rv)
    for r in range(U0.shape[0]):
        assert abs(U1[r].sum() - U0[r].sum()) < 1e-12 * max(1.0, np.abs(U0[r]).sum())


def test_fv_mhd_mass_conservation():
    cfg, prm, rv, s = orszag_tang(n=32, t_end=0.02)
    out = driver.time_integration(s, cfg, prm, rv)
    assert abs(out[0].sum() - s[0].sum()) < 1e-12 * s[0].sum()


def test_fd_interface_divergence_stays_at_roundoff():
    cfg, prm, rv, s = blast_fd(n=16, t_end=0.002)
    out = driver.time_integration(s, cfg, prm, rv)
    div = fd.interface_field_divergence(out[8], out[9], out[10], cfg.grid_spacing)
    assert np.abs(div).max() < 1e-10


def test_fd_periodic_conservation():
    """Mass and momentum are conserved to round-off.  Total energy is not
    exactly: the face-to-centre refresh of B adds 0.5 (b2_new - b2_old) to E
    (_constrained_transport.py:194-196), a non-conservative correction; its
    size here is ~1e-6 of the total."""
    cfg, prm, rv, s = blast_fd(n=16, t_end=0.002, B=(0.6, 0.5, 0.4))
    out = driver.time_integration(s, cfg, prm, rv)
    U0 = fd.cons_from_prim(s[:8], prm.gamma)
    U1 = fd.cons_from_prim(out[:8], prm.gamma)
    for r in (0, 1, 2, 3):
        assert abs(U1[r].sum() - U0[r].sum()) < 1e-11 * max(1.0, np.abs(U0[r]).sum()), r
    assert abs(U1[4].sum() - U0[4].sum()) < 1e-5 * U0[4].sum()


def test_golden_orszag_tang_summary_is_consistent():
    """The committed summary of the reference's golden file: mass = 40000 * 25/9."""
    with open(os.path.join(GOLDEN, "orszag_tang_200_t3_summary.json")) as f:
        g = json.load(f)
    assert g["sum_rho"] == pytest.approx(40000 * 25 / 9, rel=1e-14)
    assert g["shape"] == [7, 200, 200]


def test_oracle_reproduces_golden_orszag_tang():
    """200^2 Orszag-Tang on [0, 2pi]^2 to t = 3 (tests/mhd_tests/orszag_tang.py).

    Against the reference's own code run on this configuration
    (reference_orszag_tang_200_t3_summary.json, written by
    make_reference_fixtures.py --ot200): equal to round-off.  Against the
    golden file shipped with the reference (final_state_orszag_tang.npz):
    mass exactly, density to 6.9e-4 relative L1 -- the reference's own
    run misses that file by the same 6.9e-4, so the file was written by
    another revision of the scheme, not by this code."""
    with open(os.path.join(GOLDEN, "orszag_tang_200_t3_summary.json")) as f:
        g = json.load(f)
    with open(os.path.join(GOLDEN, "reference_orszag_tang_200_t3_summary.json")) as f:
        r = json.load(f)
    from astronomix_gb300 import BoundarySettings, BACKWARDS, HLL
    n, box, gamma = 200, 2 * np.pi, 5 / 3
    cfg = SimulationConfig(mhd=True, dimensionality=2, box_size=box, num_cells=n, differentiation_mode=BACKWARDS,
                           limiter=MINMOD, riemann_solver=HLL,
                           boundary_settings=BoundarySettings(*[BoundarySettings1D(2, 2)] * 3))
    rv = get_registered_variables(cfg)
    dx = box / n
    x = np.linspace(dx / 2, box - dx / 2, n)
    X, Y = np.meshgrid(x, x, indexing="ij")
    s = np.zeros((7, n, n))
    s[0], s[1], s[2], s[3] = gamma ** 2, -np.sin(Y), np.sin(X), gamma
    s[4], s[5] = -np.sin(Y), np.sin(2 * X)
    cfg = finalize_config(cfg, s.shape)
    out = driver.time_integration(s, cfg, SimulationParams(t_end=3.0, C_cfl=0.4, gamma=gamma), rv)
    # the reference's own run
    sub_r = np.asarray(r["rho_every_8"])
    assert np.abs(out[0][::8, ::8] - sub_r).max() < 1e-12 * np.abs(sub_r).max()
    for k in range(7):
        assert out[k].sum() == pytest.approx(r["row_sums"][k], rel=1e-12, abs=1e-9)
        assert out[k].min() == pytest.approx(r["row_min"][k], rel=1e-12, abs=1e-12)
        assert out[k].max() == pytest.approx(r["row_max"][k], rel=1e-12, abs=1e-12)
    # the golden file
    assert out[0].sum() == pytest.approx(g["sum_rho"], rel=1e-13)
    sub = np.asarray(g["rho_every_8"])
    l1 = np.abs(out[0][::8, ::8] - sub).sum() / np.abs(sub).sum()
    l1_ref = np.abs(sub_r - sub).sum() / np.abs(sub).sum()
    assert l1 < 1e-3 and l1 == pytest.approx(l1_ref, rel=1e-6)


def test_split_muscl_hancock_sod_vs_exact_solution():
    """The split MUSCL-Hancock scheme of the reference (evolve_state.py:52-325)
    on the Sod tube, against the exact Riemann solution."""
    from astronomix_gb300 import SPLIT, MUSCL
    cfg, prm, rv, s = sod(n=400, t_end=0.2)
    cfg = cfg._replace(split=SPLIT, time_integrator=MUSCL)
    out = driver.time_integration(s, cfg, prm, rv)
    x = (np.arange(400) + 0.5) / 400
    rho, u, p = sod_exact.sample(x, 0.2, 0.5, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1), 1.4)
    assert np.abs(out[0] - rho).sum() / 400 < 3e-3
    assert np.abs(out[2] - p).sum() / 400 < 3e-3


def test_split_scheme_conserves_on_periodic_grids():
    from astronomix_gb300 import SPLIT, MUSCL
    for dim, n in ((2, 16), (3, 8)):
        cfg, prm, rv, s = smooth_random(dim, n, seed=7, t_end=0.02)
        cfg = cfg._replace(split=SPLIT, time_integrator=MUSCL)
        out = driver.time_integration(s, cfg, prm, rv)
        U0 = fv.conserved_state_from_primitive(s, prm.gamma, dim, rv)
        U1 = fv.conserved_state_from_primitive(out, prm.gamma, dim, rv)
        for r in range(U0.shape[0]):
            assert abs(U1[r].sum() - U0[r].sum()) < 1e-12 * max(1.0, np.abs(U0[r]).sum())


def _grav_cfg(dim, boundary, dx):
    from types import SimpleNamespace
    from astronomix_gb300 import BoundarySettings, BoundarySettings1D
    b = BoundarySettings1D(boundary, boundary)
    return SimpleNamespace(dimensionality=dim, boundary_settings=b if dim == 1 else BoundarySettings(b, b, b),
                           grid_spacing=dx)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_poisson_periodic_single_mode(dim):
    """_poisson_solver.py periodic branch: lap(phi) = 4 pi G (rho - mean), so
    rho = 1 + A sin(2 pi x) gives phi = -4 pi G A sin(2 pi x) / (2 pi)^2."""
    from astronomix_gb300 import PERIODIC_BOUNDARY
    from oracle import gravity
    n = 32
    x = (np.arange(n) + 0.5) / n
    grids = np.meshgrid(*([x] * dim), indexing="ij")
    rho = 1.0 + 0.1 * np.sin(2 * np.pi * grids[0])
    phi = gravity.gravitational_potential(rho, 1.0 / n, _grav_cfg(dim, PERIODIC_BOUNDARY, 1.0 / n), 1.3)
    exact = -4 * np.pi * 1.3 * 0.1 * np.sin(2 * np.pi * grids[0]) / (2 * np.pi) ** 2
    assert np.abs(phi - exact).max() < 1e-13


def test_poisson_open_point_mass():
    """_poisson_solver.py Hockney-Eastwood branch: a unit mass in one cell has
    the isolated potential -G / r at every other cell of the grid."""
    from astronomix_gb300 import OPEN_BOUNDARY
    from oracle import gravity
    n = 24
    dx = 1.0 / n
    rho = np.zeros((n, n, n))
    rho[0, 0, 0] = 1.0 / dx ** 3
    phi = gravity.gravitational_potential(rho, dx, _grav_cfg(3, OPEN_BOUNDARY, dx), 2.0)
    i = np.arange(n) * dx
    X, Y, Z = np.meshgrid(i, i, i, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    r[0, 0, 0] = dx
    assert np.abs(phi - (-2.0 / r)).max() < 1e-12 * np.abs(phi).max()


def test_self_gravity_run_conserves_mass_and_pulls_inward():
    """A periodic over-density under self-gravity: mass is conserved to
    round-off and the gas accelerates towards the density maximum."""
    from astronomix_gb300 import DONOR_ACCOUNTING
    n = 32
    cfg, prm, rv, s = smooth_random(1, n, seed=0, t_end=0.02, amp=0.0)
    x = (np.arange(n) + 0.5) / n
    s[0] = 1.0 + 0.2 * np.cos(2 * np.pi * x)  # maximum at x = 0 (and 1)
    s[1] = 0.0
    s[2] = 1.0
    cfg = cfg._replace(self_gravity=True, self_gravity_version=DONOR_ACCOUNTING)
    prm = prm._replace(gravitational_constant=5.0)
    out = driver.time_integration(s.copy(), cfg, prm, rv)
    assert abs(out[0].sum() - s[0].sum()) < 1e-12 * s[0].sum()
    # velocity points towards x = 0 mod 1: negative on (0, 1/2), positive on (1/2, 1)
    assert out[1][2:n // 2 - 2].max() < 0 and out[1][n // 2 + 2:-2].min() > 0


def test_philox_known_answers():
    """Philox4x32-10 against the published known-answer vectors (Random123)."""
    from oracle.forcing import philox4x32_10
    cases = [((0, 0, 0, 0, 0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 6, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344, 0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for args, want in cases:
        got = tuple(int(x) for x in philox4x32_10(*args))
        assert got == want


def test_forcing_field_is_solenoidal_and_injects_edot_dt():
    """_turbulent_forcing.py: the field has no compressive part, and the
    amplitude injects exactly Edot dt of kinetic energy."""
    from types import SimpleNamespace
    from oracle import forcing
    n, box = 16, 1.0
    w = forcing.create_forcing_field(42, 3, n, box)
    k = 2 * np.pi * np.fft.fftfreq(n, d=box / n)
    kx, ky, kz = np.meshgrid(k, k, k, indexing="ij")
    wh = [np.fft.fftn(c) for c in w]
    # the real part symmetrises the spectrum; off the Nyquist planes (where
    # fftfreq gives -k for both k and -k) that keeps k . w = 0
    nyq = np.zeros((n, n, n), bool)
    nyq[n // 2], nyq[:, n // 2], nyq[:, :, n // 2] = True, True, True
    div = np.abs(np.where(nyq, 0.0, kx * wh[0] + ky * wh[1] + kz * wh[2])).max()
    assert div < 1e-10 * max(np.abs(h).max() for h in wh) * np.abs(k).max()
    cfg, prm, rv, s = smooth_random(3, n, seed=1, t_end=0.01)
    cfg = cfg._replace(num_cells=n, box_size=box, grid_spacing=box / n)
    prm = prm._replace(turbulent_forcing_params=SimpleNamespace(energy_injection_rate=3.0))
    dt = 1e-3
    out = forcing.apply_forcing(s, dt, 3, cfg, prm, rv)
    ek = lambda P: 0.5 * np.sum(P[0] * (P[1] ** 2 + P[2] ** 2 + P[3] ** 2)) * (box / n) ** 3
    assert abs((ek(out) - ek(s)) - 3.0 * dt) < 1e-10


def test_wind_source_injects_mass_loss_rate():
    """stellar_wind.py:485-584: one stage's source adds Mdot dt of mass and
    0.5 v_inf^2 Mdot dt of energy; outside 1.3 r_inj nothing changes."""
    from oracle import forcing
    n, box = 24, 1.0
    dx = box / n
    r = forcing.cell_radius(n, dx, box)
    q = np.ones((8, n, n, n))
    q[1:4] = 0.3
    src = forcing.wind_ei3d_source(q, 1e-3, 2.0, 3.0, r, dx, 4)
    assert abs(src[0].sum() * dx ** 3 - 2.0 * 1e-3) < 1e-15
    assert abs(src[4].sum() * dx ** 3 - 0.5 * 9.0 * 2.0 * 1e-3) < 1e-14
    assert np.all(src[:, r > 1.3 * 4 * dx] == 0)
