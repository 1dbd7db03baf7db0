"""Configurations and seeded initial conditions shared by the parity tests."""

import numpy as np

from astronomix_gb300 import (
    SimulationConfig, SimulationParams, BoundarySettings, BoundarySettings1D, finalize_config,
    get_registered_variables, construct_primitive_state, initialize_interface_fields,
    FINITE_DIFFERENCE, PERIODIC_BOUNDARY, OPEN_BOUNDARY, REFLECTIVE_BOUNDARY, HLL, HLLC, MINMOD,
    PERIODIC_ROLL,
)

P = PERIODIC_BOUNDARY
PERIODIC_2D = BoundarySettings(BoundarySettings1D(P, P), BoundarySettings1D(P, P), BoundarySettings1D(P, P))


def sod(n=101, dtype=np.float64, riemann=HLLC, limiter=MINMOD, t_end=0.2, C_cfl=0.8,
        boundary=(OPEN_BOUNDARY, OPEN_BOUNDARY)):
    """1D Sod shock tube on [0, 1] (gamma 1.4)."""
    cfg = SimulationConfig(dimensionality=1, box_size=1.0, num_cells=n, riemann_solver=riemann, limiter=limiter,
                           boundary_settings=BoundarySettings1D(*boundary))
    rv = get_registered_variables(cfg)
    dx = 1.0 / n
    x = np.linspace(dx / 2, 1 - dx / 2, n)
    rho = np.where(x < 0.5, 1.0, 0.125).astype(dtype)
    p = np.where(x < 0.5, 1.0, 0.1).astype(dtype)
    u = np.zeros(n, dtype=dtype)
    s = construct_primitive_state(cfg, rv, density=rho, velocity_x=u, gas_pressure=p)
    cfg = finalize_config(cfg, s.shape)
    prm = SimulationParams(C_cfl=C_cfl, gamma=1.4, t_end=t_end)
    return cfg, prm, rv, s


def orszag_tang(n=64, dtype=np.float64, t_end=0.01, riemann=HLL, C_cfl=0.4, roll=False, limiter=MINMOD,
                boundary=None):
    """2D Orszag-Tang vortex on [0,1]^2, gamma 5/3 (rho=25/(36 pi), p=5/(12 pi));
    `boundary`: one code for every side instead of periodic."""
    bs = PERIODIC_2D if boundary is None else BoundarySettings(*[BoundarySettings1D(boundary, boundary)] * 3)
    cfg = SimulationConfig(mhd=True, dimensionality=2, box_size=1.0, num_cells=n, riemann_solver=riemann,
                           limiter=limiter, boundary_settings=bs,
                           boundary_handling=PERIODIC_ROLL if roll else 0)
    rv = get_registered_variables(cfg)
    dx = 1.0 / n
    x = (np.arange(n) + 0.5) * dx
    X, Y = np.meshgrid(x, x, indexing="ij")
    rho = np.full_like(X, 25 / (36 * np.pi))
    p = np.full_like(X, 5 / (12 * np.pi))
    vx, vy = -np.sin(2 * np.pi * Y), np.sin(2 * np.pi * X)
    B0 = 1 / np.sqrt(4 * np.pi)
    bx, by = -B0 * np.sin(2 * np.pi * Y), B0 * np.sin(4 * np.pi * X)
    s = construct_primitive_state(cfg, rv, density=rho.astype(dtype), velocity_x=vx, velocity_y=vy,
                                  magnetic_field_x=bx, magnetic_field_y=by, magnetic_field_z=np.zeros_like(X),
                                  gas_pressure=p)
    cfg = finalize_config(cfg, s.shape)
    prm = SimulationParams(C_cfl=C_cfl, gamma=5 / 3, t_end=t_end)
    return cfg, prm, rv, s


def smooth_random(dim, n, seed, dtype=np.float64, mhd=False, riemann=HLL, limiter=MINMOD, t_end=0.01,
                  boundary=P, roll=False, amp=0.2):
    """Seeded smooth random fields (sums of a few Fourier modes) on a periodic box."""
    rng = np.random.default_rng(seed)
    bs = BoundarySettings(*[BoundarySettings1D(boundary, boundary)] * 3) if dim > 1 else \
        BoundarySettings1D(boundary, boundary)
    cfg = SimulationConfig(mhd=mhd, dimensionality=dim, box_size=1.0, num_cells=n, riemann_solver=riemann,
                           limiter=limiter, boundary_settings=bs, boundary_handling=PERIODIC_ROLL if roll else 0)
    rv = get_registered_variables(cfg)
    x = (np.arange(n) + 0.5) / n
    grids = np.meshgrid(*([x] * dim), indexing="ij")

    def field(base, a):
        f = np.full(grids[0].shape, base)
        for _ in range(3):
            k = rng.integers(1, 3, size=dim)
            ph = rng.uniform(0, 2 * np.pi)
            f = f + a * rng.uniform(-1, 1) * np.sin(2 * np.pi * sum(ki * g for ki, g in zip(k, grids)) + ph)
        return f

    rho = field(1.0, amp)
    p = field(1.0, amp)
    v = [field(0.0, 0.5) for _ in range(dim)]
    kw = dict(density=rho.astype(dtype), gas_pressure=p, velocity_x=v[0])
    if dim >= 2:
        kw["velocity_y"] = v[1]
    if dim == 3:
        kw["velocity_z"] = v[2]
    if mhd:
        kw.update(magnetic_field_x=field(0.3, 0.2), magnetic_field_y=field(0.1, 0.2),
                  magnetic_field_z=field(0.0, 0.2) if dim == 3 else np.zeros_like(rho))
    s = construct_primitive_state(cfg, rv, **kw)
    cfg = finalize_config(cfg, s.shape)
    prm = SimulationParams(C_cfl=0.4, gamma=5 / 3, t_end=t_end)
    return cfg, prm, rv, s


def blast_fd(n=32, dtype=np.float64, t_end=0.002, C_cfl=1.5, p_in=10.0, p_out=0.1, r0=0.1,
             rhomin=1e-14, pmin=1e-14, B=(1 / np.sqrt(2), 1 / np.sqrt(2), 0.0)):
    """3D MHD blast for the finite-difference scheme (periodic unit cube)."""
    cfg = SimulationConfig(solver_mode=FINITE_DIFFERENCE, mhd=True, dimensionality=3, box_size=1.0,
                           num_cells=n, boundary_settings=PERIODIC_2D, boundary_handling=PERIODIC_ROLL)
    rv = get_registered_variables(cfg)
    x = (np.arange(n) + 0.5) / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2)
    rho = np.ones_like(X)
    p = np.where(r < r0, p_in, p_out)
    bx = np.full_like(X, B[0])
    by = np.full_like(X, B[1])
    bz = np.full_like(X, B[2])
    fx, fy, fz = initialize_interface_fields(bx, by, bz)
    z = np.zeros_like(X)
    s = construct_primitive_state(cfg, rv, density=rho.astype(dtype), velocity_x=z, velocity_y=z, velocity_z=z,
                                  magnetic_field_x=bx, magnetic_field_y=by, magnetic_field_z=bz,
                                  interface_magnetic_field_x=fx, interface_magnetic_field_y=fy,
                                  interface_magnetic_field_z=fz, gas_pressure=p)
    cfg = finalize_config(cfg, s.shape)
    prm = SimulationParams(C_cfl=C_cfl, gamma=5 / 3, t_end=t_end, minimum_density=rhomin, minimum_pressure=pmin)
    return cfg, prm, rv, s


def _groups(nrows):
    """Rows sharing one scale: density, velocity vector, pressure, magnetic field (cell and face)."""
    return {3: [[0], [1], [2]], 4: [[0], [1, 2], [3]], 5: [[0], [1, 2, 3], [4]],
            7: [[0], [1, 2], [3], [4, 5, 6]], 8: [[0], [1, 2, 3], [4], [5, 6, 7]],
            11: [[0], [1, 2, 3], [4], [5, 6, 7, 8, 9, 10]]}.get(nrows, [[i] for i in range(nrows)])


def rel_err(a, b):
    """max over rows of max|a-b| / scale, the scale being max|b| over the row's group
    (a vector component that is zero in exact arithmetic is measured against its vector)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    out = 0.0
    for grp in _groups(b.shape[0]):
        scale = max(max(np.abs(b[i]).max() for i in grp), 1e-300)
        for i in grp:
            out = max(out, np.abs(a[i] - b[i]).max() / scale)
    return out


def rel_l1(a, b, row=0):
    a = np.asarray(a, dtype=np.float64)[row]
    b = np.asarray(b, dtype=np.float64)[row]
    return np.abs(a - b).sum() / np.abs(b).sum()
