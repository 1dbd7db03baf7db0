"""Writes tests/golden/reference_fixtures.npz: results of the reference's own code.

Imports leo1200/astronomix unchanged from a source tree (first argument, or
the AMX_REFERENCE_PATH environment variable) on the NumPy stand-ins for jax,
jaxtyping, beartype, equinox and astropy in tests/golden/jaxshim/, and runs
the cases of reference_cases.py in float64: whole `time_integration` calls
(RUN_CASES) and single hot-path functions on seeded inputs (SEAM_CASES).
Bytecode writing is off, so nothing is written into the reference tree.
Run from the repository root:

    python tests/golden/make_reference_fixtures.py /path/to/astronomix-checkout [--ot200]

--ot200 also runs tests/mhd_tests/orszag_tang.py's configuration (200^2 on
[0, 2 pi]^2 to t = 3, about 1000 steps) and writes its summary to
reference_orszag_tang_200_t3_summary.json.
"""
import hashlib
import json
import os
import sys
import time

sys.dont_write_bytecode = True

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _import_reference(path):
    sys.path.insert(0, os.path.join(HERE, "jaxshim"))
    sys.path.insert(0, path)
    import astronomix  # noqa: F401
    return astronomix


def digest(a):
    import numpy as np
    return hashlib.sha256(np.ascontiguousarray(np.asarray(a, dtype=np.float64)).tobytes()).hexdigest()[:16]


def to_reference(obj, classes):
    """This package's option NamedTuples -> the reference's classes of the same name."""
    if isinstance(obj, tuple) and hasattr(obj, "_fields"):
        cls = classes.get(type(obj).__name__)
        vals = {k: to_reference(v, classes) for k, v in obj._asdict().items()}
        if cls is None:
            return type(obj)(**vals)
        return cls(**{k: v for k, v in vals.items() if k in cls._fields})
    return obj


def reference_classes():
    import importlib
    out = {}
    for mod in ("astronomix.option_classes.simulation_config", "astronomix.option_classes.simulation_params",
                "astronomix._physics_modules._stellar_wind.stellar_wind_options",
                "astronomix._physics_modules._turbulent_forcing._turbulent_forcing_options",
                "astronomix._physics_modules._cosmic_rays.cosmic_ray_options",
                "astronomix._physics_modules._cooling.cooling_options",
                "astronomix._physics_modules._neural_net_force._neural_net_force_options",
                "astronomix._physics_modules._cnn_mhd_corrector._cnn_mhd_corrector_options"):
        m = importlib.import_module(mod)
        for name in dir(m):
            v = getattr(m, name)
            if isinstance(v, type) and issubclass(v, tuple) and hasattr(v, "_fields"):
                out.setdefault(name, v)
    return out


def run_cases(ax, classes):
    import numpy as np
    from reference_cases import RUN_CASES
    from astronomix.option_classes.simulation_config import finalize_config as ref_finalize
    from astronomix.variable_registry.registered_variables import get_registered_variables as ref_rv

    out = {}
    for name, make in RUN_CASES.items():
        cfg, prm, rv, s = make()
        rcfg = to_reference(cfg, classes)
        # the reference's finalize_config must leave the converted (already finalised) config as it is
        again = ref_finalize(rcfg, s.shape)
        assert again == rcfg, name
        rprm = to_reference(prm, classes)
        rrv = ref_rv(rcfg)
        assert tuple(rrv) == tuple(to_reference(rv, classes)), name
        t0 = time.time()
        res = np.asarray(ax.time_integration(np.array(s, dtype=np.float64), rcfg, rprm, rrv), dtype=np.float64)
        out[name + "/output"] = res
        out[name + "/input_digest"] = np.array(digest(s))
        print("%-32s %6.2f s" % (name, time.time() - t0), flush=True)
    return out


def seam_cases(classes):
    import numpy as np
    import reference_cases as rc
    from astronomix_gb300 import (SimulationConfig, SimulationParams, finalize_config, get_registered_variables,
                                  HLL, HLLC, HLLC_LM, LAX_FRIEDRICHS, AM_HLLC, HYBRID_HLLC, MINMOD, OSHER,
                                  DOUBLE_MINMOD, SUPERBEE,
                                  VAN_ALBADA, PERIODIC_ROLL, FINITE_DIFFERENCE)
    from _cases import PERIODIC_2D
    from astronomix._finite_volume._riemann_solver._riemann_solver import _riemann_solver
    from astronomix._finite_volume._state_evolution.limited_gradients import _calculate_limited_gradients
    from astronomix._finite_volume._magnetic_update._magnetic_field_update import magnetic_update
    from astronomix._finite_volume._timestep_estimation._timestep_estimator import _cfl_time_step
    from astronomix._finite_difference._timestep_estimation._timestep_estimator import _cfl_time_step_fd
    from astronomix._finite_difference._interface_fluxes._weno import _weno_flux_x, _weno_flux_y, _weno_flux_z
    from astronomix._finite_difference._fluid_equations._eigen import _eigen_all_lambdas
    from astronomix._finite_difference._magnetic_update._constrained_transport import (
        constrained_transport_rhs, update_cell_center_fields)
    from astronomix._finite_difference._fluid_equations._enforce_positivity import _enforce_positivity
    from astronomix._finite_difference._state_evolution._evolve_state import _evolve_state_fd
    from astronomix.data_classes.simulation_helper_data import get_helper_data
    from astronomix.variable_registry.registered_variables import get_registered_variables as ref_rv
    from oracle import fd as ofd

    def hydro2d(riemann=HLL, limiter=MINMOD, n=16):
        cfg = SimulationConfig(dimensionality=2, box_size=1.0, num_cells=n, riemann_solver=riemann, limiter=limiter,
                               boundary_settings=PERIODIC_2D, boundary_handling=PERIODIC_ROLL)
        cfg = finalize_config(cfg, (4, n, n))
        rcfg = to_reference(cfg, classes)
        return cfg, rcfg, ref_rv(rcfg)

    def mhd3d(n=8):
        cfg = SimulationConfig(solver_mode=FINITE_DIFFERENCE, mhd=True, dimensionality=3, box_size=1.0,
                               num_cells=n, boundary_settings=PERIODIC_2D, boundary_handling=PERIODIC_ROLL)
        cfg = finalize_config(cfg, (11, n, n, n))
        rcfg = to_reference(cfg, classes)
        return cfg, rcfg, ref_rv(rcfg)

    g = 5 / 3
    out = {}
    PL, PR, P3 = rc.prim2d(1), rc.prim2d(2), rc.prim2d(3)
    for name, rs, d in (("riemann_hll", HLL, 1), ("riemann_hllc", HLLC, 2), ("riemann_hllc_lm", HLLC_LM, 1),
                        ("riemann_lax_friedrichs", LAX_FRIEDRICHS, 1), ("riemann_am_hllc", AM_HLLC, 1),
                        ("riemann_hybrid_hllc", HYBRID_HLLC, 2)):
        cfg, rcfg, rrv = hydro2d(riemann=rs)
        out[name + "/output"] = np.asarray(_riemann_solver(PL, PR, P3, g, rcfg, rrv, d))
    P = rc.prim2d(4)
    grads = []
    for lim in (MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA):
        cfg, rcfg, rrv = hydro2d(limiter=lim)
        hd = get_helper_data(rcfg)
        for axis in (1, 2):
            grads.append(np.asarray(_calculate_limited_gradients(P, rcfg, hd, axis)))
    out["limited_gradients/output"] = np.stack(grads)
    # magnetic update: 2D MHD, periodic roll
    cfg = SimulationConfig(mhd=True, dimensionality=2, box_size=1.0, num_cells=16, riemann_solver=HLL,
                           boundary_settings=PERIODIC_2D, boundary_handling=PERIODIC_ROLL)
    cfg = finalize_config(cfg, (7, 16, 16))
    rcfg = to_reference(cfg, classes)
    rrv = ref_rv(rcfg)
    B, gas = rc.mag2d(5)
    Bn, gn = magnetic_update(B, gas, cfg.grid_spacing, 1e-3, rrv, rcfg)
    out["magnetic_update_2d/output"] = np.concatenate([np.asarray(gn), np.asarray(Bn)])
    cfg, rcfg, rrv = hydro2d()
    out["cfl_fv_2d/output"] = np.array(float(_cfl_time_step(rc.prim2d(6), cfg.grid_spacing, 1.0, g, rcfg, rrv, 0.4)))
    # FD
    cfg, rcfg, rrv = mhd3d()
    rprm = to_reference(SimulationParams(C_cfl=1.5, gamma=g, minimum_density=1e-14, minimum_pressure=1e-14), classes)
    U = rc.cons3d_mhd(7)
    Pfd = ofd.prim_from_cons(U, 1e-14, 1e-14, g)
    out["cfl_fd/output"] = np.array(float(_cfl_time_step_fd(Pfd, cfg.grid_spacing, 1.0, g, rcfg, rprm, rrv, 1.5)))
    U = rc.cons3d_mhd(8)
    out["weno_flux/output"] = np.stack([np.asarray(f(U, 1e-14, 1e-14, g, rcfg, rrv))
                                        for f in (_weno_flux_x, _weno_flux_y, _weno_flux_z)])
    out["eigen_lambdas/output"] = np.asarray(_eigen_all_lambdas(rc.cons3d_mhd(9), 1e-14, 1e-14, g, rrv))
    U = rc.cons3d_mhd(10)
    Fx, Fy, Fz = rc.fluxes3d(10)
    dtdx = 0.01
    rb = constrained_transport_rhs(U, Fx, Fy, Fz, dtdx, dtdx, dtdx, rrv)
    out["constrained_transport_rhs/output"] = np.stack([np.asarray(v) for v in rb])
    out["enforce_positivity/output"] = np.asarray(_enforce_positivity(rc.cons3d_mhd(11), g, 1.1, 0.9, rrv))
    bx, by, bz = rc.faces3d(12)
    out["update_cell_center_fields/output"] = np.asarray(update_cell_center_fields(rc.cons3d_mhd(12), bx, by, bz,
                                                                                   rrv))
    U = rc.cons3d_mhd(13)
    bx, by, bz = rc.faces3d(13)
    Pst = np.concatenate([ofd.prim_from_cons(U, 1e-14, 1e-14, g), np.stack([bx, by, bz])])
    hd = get_helper_data(rcfg)
    out["evolve_state_fd/output"] = np.asarray(_evolve_state_fd(Pst, 2e-3, g, 1.0, rcfg, rprm, hd, rrv))
    return out


def ot200(ax, classes):
    import numpy as np
    from astronomix_gb300 import (SimulationConfig, SimulationParams, BoundarySettings, BoundarySettings1D,
                                  finalize_config, get_registered_variables, BACKWARDS, HLL, MINMOD)
    from astronomix.variable_registry.registered_variables import get_registered_variables as ref_rv

    n, box, gamma = 200, 2 * np.pi, 5 / 3
    cfg = SimulationConfig(mhd=True, dimensionality=2, box_size=box, num_cells=n, differentiation_mode=BACKWARDS,
                           limiter=MINMOD, riemann_solver=HLL,
                           boundary_settings=BoundarySettings(*[BoundarySettings1D(2, 2)] * 3))
    dx = box / n
    x = np.linspace(dx / 2, box - dx / 2, n)
    X, Y = np.meshgrid(x, x, indexing="ij")
    s = np.zeros((7, n, n))
    s[0], s[1], s[2], s[3] = gamma ** 2, -np.sin(Y), np.sin(X), gamma
    s[4], s[5] = -np.sin(Y), np.sin(2 * X)
    cfg = finalize_config(cfg, s.shape)
    rcfg = to_reference(cfg, classes)
    t0 = time.time()
    g = np.asarray(ax.time_integration(s, rcfg, to_reference(SimulationParams(t_end=3.0, C_cfl=0.4, gamma=gamma),
                                                             classes), ref_rv(rcfg)))
    print("orszag_tang_200_t3 %.1f s" % (time.time() - t0), flush=True)
    return {
        "source": "leo1200/astronomix time_integration run by make_reference_fixtures.py (NumPy stand-in for JAX)",
        "shape": list(g.shape),
        "sum_rho": float(g[0].sum()),
        "row_sums": [float(v) for v in g.reshape(g.shape[0], -1).sum(1)],
        "row_min": [float(v) for v in g.reshape(g.shape[0], -1).min(1)],
        "row_max": [float(v) for v in g.reshape(g.shape[0], -1).max(1)],
        "rho_every_8": g[0][::8, ::8].tolist(),
    }


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    path = args[0] if args else os.environ.get("AMX_REFERENCE_PATH")
    if not path:
        sys.exit("usage: make_reference_fixtures.py <reference source tree> [--ot200]")
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, HERE)
    import numpy as np
    ax = _import_reference(path)
    classes = reference_classes()
    out = run_cases(ax, classes)
    out.update(seam_cases(classes))
    np.savez_compressed(os.path.join(HERE, "reference_fixtures.npz"), **out)
    if "--ot200" in sys.argv:
        with open(os.path.join(HERE, "reference_orszag_tang_200_t3_summary.json"), "w") as f:
            json.dump(ot200(ax, classes), f)


if __name__ == "__main__":
    main()
