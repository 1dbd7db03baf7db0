"""Seeded cases whose results the reference itself computed (tests/golden/reference_fixtures.npz).

Shared by make_reference_fixtures.py, which runs them through leo1200/astronomix
(imported unchanged on a NumPy stand-in for JAX), and by the tests that hold
the oracle and the CUDA path against the stored results.  Every case is
built with this package's mirror of the reference's option classes; the
generator converts the NamedTuples to the reference's own classes by name.

RUN_CASES: ``time_integration(state, config, params, registered_variables)``
(time_stepping/time_integration.py:61-236), FP64, the final state stored.

SEAM_CASES: single hot-path functions on seeded random inputs: the Riemann
solvers, the limited gradients, the magnetic update, both CFL estimates, the
WENO fluxes, the eigenvalues, constrained transport, the positivity floors,
the cell-centre field refresh, one FD step.
"""

import numpy as np

from astronomix_gb300 import (
    HLL, HLLC, HLLC_LM, LAX_FRIEDRICHS, HYBRID_HLLC, AM_HLLC, MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA, VAN_ALBADA_PP,
    OPEN_BOUNDARY, REFLECTIVE_BOUNDARY, PERIODIC_BOUNDARY, SPLIT, MUSCL, IMPLICIT_EULER,
)

from _cases import sod, orszag_tang, smooth_random, blast_fd


def _floored_blast(n=12):
    cfg, prm, rv, s = blast_fd(n=n, t_end=0.003, B=(0.6, 0.5, 0.4), rhomin=0.5, pmin=0.2)
    x = (np.arange(n) + 0.5) / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    blob = (X - 0.25) ** 2 + (Y - 0.3) ** 2 + (Z - 0.7) ** 2 < 0.2 ** 2
    s = s.copy()
    s[0] = np.where(blob, 0.3, s[0])
    return cfg, prm, rv, s


def _split(case):
    cfg, prm, rv, s = case
    return cfg._replace(split=SPLIT, time_integrator=MUSCL), prm, rv, s


def _mixed():
    """x reflective on the left and open on the right, y reflective on both sides."""
    from astronomix_gb300 import BoundarySettings, BoundarySettings1D
    return BoundarySettings(BoundarySettings1D(REFLECTIVE_BOUNDARY, OPEN_BOUNDARY),
                            BoundarySettings1D(REFLECTIVE_BOUNDARY, REFLECTIVE_BOUNDARY),
                            BoundarySettings1D(REFLECTIVE_BOUNDARY, REFLECTIVE_BOUNDARY))


def _with(case, **kw):
    cfg, prm, rv, s = case
    return cfg._replace(**kw), prm, rv, s


RUN_CASES = {
    # configuration 1 as specified: Sod, HLLC, MINMOD, 101 cells, C_cfl 0.8, t_end 0.2
    "sod_hllc_t02": lambda: sod(riemann=HLLC, t_end=0.2),
    "sod_hll": lambda: sod(riemann=HLL, t_end=0.05),
    "sod_hllc_lm": lambda: sod(riemann=HLLC_LM, t_end=0.05),
    "sod_lax_friedrichs": lambda: sod(riemann=LAX_FRIEDRICHS, t_end=0.05),
    "sod_osher": lambda: sod(limiter=OSHER, t_end=0.03),
    "sod_double_minmod": lambda: sod(limiter=DOUBLE_MINMOD, t_end=0.03),
    "sod_superbee": lambda: sod(limiter=SUPERBEE, t_end=0.03),
    "sod_van_albada": lambda: sod(limiter=VAN_ALBADA, t_end=0.03),
    "sod_reflective": lambda: sod(boundary=(REFLECTIVE_BOUNDARY, REFLECTIVE_BOUNDARY), t_end=0.15),
    "sod_periodic": lambda: sod(boundary=(PERIODIC_BOUNDARY, PERIODIC_BOUNDARY), t_end=0.15),
    "sod_split": lambda: _split(sod(riemann=HLLC, t_end=0.1)),
    "hydro2d_hllc": lambda: smooth_random(2, 24, seed=21, riemann=HLLC, t_end=0.01),
    "hydro2d_open": lambda: smooth_random(2, 20, seed=7, boundary=OPEN_BOUNDARY, t_end=0.01),
    "hydro2d_reflective": lambda: smooth_random(2, 20, seed=7, boundary=REFLECTIVE_BOUNDARY, t_end=0.01),
    "hydro2d_van_albada_pp": lambda: smooth_random(2, 20, seed=9, limiter=VAN_ALBADA_PP, t_end=0.01),
    "hydro3d_lax_friedrichs": lambda: smooth_random(3, 12, seed=33, riemann=LAX_FRIEDRICHS, t_end=0.01),
    "ot32_hll": lambda: orszag_tang(n=32, t_end=0.01),
    "ot32_hllc_roll": lambda: orszag_tang(n=32, t_end=0.01, roll=True, riemann=HLLC),
    "ot32_euler": lambda: _with(orszag_tang(n=32, t_end=0.01), fv_magnetic_integrator=IMPLICIT_EULER),
    "ot32_split": lambda: _split(orszag_tang(n=32, t_end=0.01, riemann=HLLC)),
    "mhd2d_van_albada_pp": lambda: smooth_random(2, 20, seed=19, mhd=True, limiter=VAN_ALBADA_PP, t_end=0.005),
    "mhd3d_hll": lambda: smooth_random(3, 12, seed=3, mhd=True, t_end=0.005),
    "mhd3d_lax_friedrichs": lambda: smooth_random(3, 12, seed=3, mhd=True, riemann=LAX_FRIEDRICHS, t_end=0.005),
    "sod_am_hllc": lambda: sod(riemann=AM_HLLC, t_end=0.1),
    "sod_hybrid_hllc": lambda: sod(riemann=HYBRID_HLLC, t_end=0.1),
    "hydro2d_am_hllc": lambda: smooth_random(2, 24, seed=23, riemann=AM_HLLC, t_end=0.02, amp=0.5),
    "hydro3d_hybrid_hllc": lambda: smooth_random(3, 12, seed=24, riemann=HYBRID_HLLC, t_end=0.02, amp=0.5),
    "ot32_am_hllc": lambda: orszag_tang(n=32, t_end=0.02, riemann=AM_HLLC),
    # the split sweeps with the compression switch (evolve_state.py:80-88 passes the sweep's state)
    "sod_split_am_hllc": lambda: _split(sod(riemann=AM_HLLC, t_end=0.1)),
    "hydro2d_split_hybrid_hllc": lambda: _split(smooth_random(2, 24, seed=25, riemann=HYBRID_HLLC, t_end=0.02,
                                                              amp=0.5)),
    "hydro2d_split_am_hllc_reflective": lambda: _split(smooth_random(2, 20, seed=27, riemann=AM_HLLC, t_end=0.02,
                                                                     amp=0.5, boundary=REFLECTIVE_BOUNDARY)),
    "hydro3d_split_am_hllc_open": lambda: _split(smooth_random(3, 12, seed=26, riemann=AM_HLLC, t_end=0.01, amp=0.5,
                                                               boundary=OPEN_BOUNDARY)),
    "ot32_split_am_hllc": lambda: _split(orszag_tang(n=32, t_end=0.02, riemann=AM_HLLC)),
    "ot32_reflective": lambda: orszag_tang(n=32, t_end=0.02, boundary=REFLECTIVE_BOUNDARY),
    # 3D MHD with reflective walls: the 3-vectors of the magnetic update negate
    # y at x walls, z at y walls, and nothing at z walls (a dropped update)
    "mhd3d_reflective": lambda: smooth_random(3, 12, seed=31, mhd=True, t_end=0.006, boundary=REFLECTIVE_BOUNDARY),
    "mhd3d_split_reflective_open": lambda: _split(_with(smooth_random(3, 10, seed=32, mhd=True, riemann=HLLC,
                                                                      t_end=0.006, boundary=REFLECTIVE_BOUNDARY),
                                                        boundary_settings=_mixed())),
    "mhd2d_reflective_open": lambda: _with(smooth_random(2, 24, seed=29, mhd=True, t_end=0.01,
                                                         boundary=REFLECTIVE_BOUNDARY), boundary_settings=_mixed()),
    "fd_blast12_oblique": lambda: blast_fd(n=12, t_end=0.003, B=(0.6, 0.5, 0.4)),
    "fd_blast12_floors": lambda: _floored_blast(12),
    "fd_blast12_zero_normal_field": lambda: blast_fd(n=12, t_end=0.003),
}


def _rng(seed):
    return np.random.default_rng(seed)


def prim2d(seed, n=16):
    """A random 2D hydro primitive state (rho, vx, vy, p), positive rho and p."""
    r = _rng(seed)
    P = np.empty((4, n, n))
    P[0] = 1.0 + 0.5 * r.random((n, n))
    P[1:3] = r.standard_normal((2, n, n))
    P[3] = 0.5 + r.random((n, n))
    return P


def cons3d_mhd(seed, n=8, B=(0.6, 0.5, 0.4)):
    """A random 3D MHD conserved state of the FD scheme (8 rows)."""
    r = _rng(seed)
    rho = 1.0 + 0.3 * r.random((n, n, n))
    v = 0.5 * r.standard_normal((3, n, n, n))
    Bc = np.array(B)[:, None, None, None] + 0.2 * r.standard_normal((3, n, n, n))
    p = 0.5 + r.random((n, n, n))
    U = np.empty((8, n, n, n))
    U[0] = rho
    U[1:4] = rho * v
    U[4] = p / (5 / 3 - 1) + 0.5 * rho * (v ** 2).sum(0) + 0.5 * (Bc ** 2).sum(0)
    U[5:8] = Bc
    return U


def faces3d(seed, n=8):
    return [0.6 + 0.2 * _rng(seed + k).standard_normal((n, n, n)) for k in range(3)]


def fluxes3d(seed, n=8):
    return [0.3 * _rng(seed + 10 + k).standard_normal((8, n, n, n)) for k in range(3)]


def mag2d(seed, n=16):
    """B (3 rows) and the 2D MHD gas state (rho, vx, vy, p) for magnetic_update."""
    r = _rng(seed)
    B = 0.5 * r.standard_normal((3, n, n))
    gas = prim2d(seed + 1, n)
    return B, gas


# name -> description; the inputs are the seeded helpers above
SEAM_CASES = {
    "riemann_hll": "Riemann solver HLL on prim2d(1) | prim2d(2), axis 1 (x)",
    "riemann_hllc": "HLLC, axis 2",
    "riemann_hllc_lm": "HLLC-LM, axis 1",
    "riemann_lax_friedrichs": "Lax-Friedrichs (global alpha over prim2d(3)), axis 1",
    "riemann_am_hllc": "AM-HLLC (compression switch from prim2d(3)), axis 1",
    "riemann_hybrid_hllc": "HYBRID_HLLC, axis 2",
    "limited_gradients": "limited gradients of prim2d(4) along axis 1 and 2 for every limiter",
    "magnetic_update_2d": "magnetic_update of mag2d(5), dt 1e-3, periodic roll",
    "cfl_fv_2d": "_cfl_time_step (UNSPLIT) of prim2d(6)",
    "cfl_fd": "_cfl_time_step_fd of the primitive form of cons3d_mhd(7)",
    "weno_flux": "_weno_flux_x / _y / _z of cons3d_mhd(8)",
    "eigen_lambdas": "_eigen_all_lambdas of cons3d_mhd(9)",
    "constrained_transport_rhs": "constrained_transport_rhs of cons3d_mhd(10), fluxes3d(10)",
    "enforce_positivity": "_enforce_positivity of cons3d_mhd(11) with floors 1.1 / 0.9",
    "update_cell_center_fields": "update_cell_center_fields of cons3d_mhd(12), faces3d(12)",
    "evolve_state_fd": "_evolve_state_fd of cons3d_mhd(13) (as primitives + faces), dt 2e-3",
}
