"""Oracle: self-gravity of the finite-volume scheme (test infrastructure only).

Nothing in the product imports this module; it is the checker the CUDA
gravity kernels are compared against.  It restates, operation for operation,
astronomix 0.5.1's

* ``_physics_modules/_self_gravity/_poisson_solver.py:17-151``
  (``_compute_gravitational_potential``: periodic FFT solve with the mean
  subtracted, or the Hockney-Eastwood zero-padded convolution for open
  boundaries), and
* ``_physics_modules/_self_gravity/_self_gravity.py:68-390``
  (``_gravitational_source_term_along_axis`` in its five versions and
  ``_apply_self_gravity``),

on the padded arrays the reference holds (so with ghost cells the FFT runs
over the padded grid, as the reference's does).  NumPy only: the FFTs are
``numpy.fft``'s, the same transforms as ``jax.numpy.fft``.
"""

import numpy as np

from astronomix_gb300.option_classes import (
    PERIODIC_BOUNDARY, SIMPLE_SOURCE_TERM, DONOR_ACCOUNTING, RIEMANN_SPLIT,
    RIEMANN_SPLIT_UNSTABLE, HALF_SPLIT, HLLC, HLLC_LM, SPLIT, UNSPLIT, GHOST_CELLS,
)
from . import fv as _fv


def all_periodic(config):
    """_poisson_solver.py:39-79: periodic only if every boundary is."""
    bs = config.boundary_settings
    if config.dimensionality == 1:
        return bs.left_boundary == PERIODIC_BOUNDARY and bs.right_boundary == PERIODIC_BOUNDARY
    axes = [bs.x, bs.y, bs.z][:config.dimensionality]
    return all(b.left_boundary == PERIODIC_BOUNDARY and b.right_boundary == PERIODIC_BOUNDARY for b in axes)


def gravitational_potential(rho, grid_spacing, config, G=1.0):
    """_poisson_solver.py:17-151 on the array it is given (padded or not)."""
    rho = np.asarray(rho)
    d = config.dimensionality
    dtype = rho.dtype
    if all_periodic(config):
        rho = rho - np.mean(rho)
        rho_k = np.fft.fftn(rho)
        n = rho.shape[0]
        k_base = np.fft.fftfreq(n, d=grid_spacing) * 2 * np.pi
        if d == 1:
            k2 = k_base ** 2
        elif d == 2:
            kx, ky = np.meshgrid(k_base, k_base, indexing="ij")
            k2 = kx ** 2 + ky ** 2
        else:
            kx, ky, kz = np.meshgrid(k_base, k_base, k_base, indexing="ij")
            k2 = kx ** 2 + ky ** 2 + kz ** 2
        k2 = np.where(k2 == 0, 1e-12, k2)
        green = np.where(k2 > 1e-12, -4 * np.pi * G / k2, -1 / (4 * np.pi))
        return np.real(np.fft.ifftn(green * rho_k)).astype(dtype)
    # Hockney & Eastwood: zero-padded to twice the size, isolated kernel
    shape = rho.shape
    ext = np.zeros(tuple(2 * s for s in shape), dtype=dtype)
    sl = tuple(slice(0, s) for s in shape)
    ext[sl] = rho
    grids = []
    for n in shape:
        pos = np.arange(2 * n)
        pos = np.where(pos < n, pos, 2 * n - pos) * grid_spacing
        grids.append(pos)
    if d == 1:
        r = grids[0]
    elif d == 2:
        x, y = np.meshgrid(grids[0], grids[1], indexing="ij")
        r = np.sqrt(x ** 2 + y ** 2)
    else:
        x, y, z = np.meshgrid(grids[0], grids[1], grids[2], indexing="ij")
        r = np.sqrt(x ** 2 + y ** 2 + z ** 2)
    r_safe = np.where(r == 0, grid_spacing, r)
    if d == 1:
        kern = -2 * np.pi * G * r
    elif d == 2:
        kern = -2 * G * np.log(r_safe)
    else:
        kern = -G / r_safe
    pot = np.real(np.fft.ifftn(np.fft.fftn(ext) * np.fft.fftn(kern)))[sl]
    return (pot * grid_spacing ** d).astype(dtype)


def _stencil_diff(phi, hi, lo, axis):
    """_stencil_operations.py:33-58 with factors (1, -1): phi[i+hi] - phi[i+lo]."""
    return np.roll(phi, -hi, axis) + (-1.0) * np.roll(phi, -lo, axis)


def _interface_states(P, dt, gamma, config, rv, axis, C_cfl=None):
    """_self_gravity.py:125-158: the interface states of the old state."""
    if config.first_order_fallback:
        return np.roll(P, 1, axis), P
    if config.split == SPLIT:
        return _fv.reconstruct_split(P, dt, gamma, config, rv, axis)
    # the unsplit reconstruction of every axis; only `axis` is used
    return _fv.reconstruct_unsplit_single(P, config, axis)


def _riemann_split_fluxes(PL, PR, gamma, config, rv, axis):
    """_self_gravity.py:159-284: HLLC with the dissipation split between the
    two cells of every interface; returns (what cell i accounts for towards
    i-1, what cell i-1 accounts for), both at the interface between i-1 and i."""
    if config.riemann_solver not in (HLLC, HLLC_LM):
        raise NotImplementedError("The RIEMANN_SPLIT gravity scheme is currently only implemented for HLLC and HLLC_LM.")
    dims = config.dimensionality
    rhoL, uL, pL = PL[rv.density_index], PL[axis], PL[rv.pressure_index]
    rhoR, uR, pR = PR[rv.density_index], PR[axis], PR[rv.pressure_index]
    cL = _fv.speed_of_sound(rhoL, pL, gamma)
    cR = _fv.speed_of_sound(rhoR, pR, gamma)
    FL = _fv.euler_flux(PL, gamma, dims, rv, axis)
    FR = _fv.euler_flux(PR, gamma, dims, rv, axis)
    u_hat = (np.sqrt(rhoL) * uL + np.sqrt(rhoR) * uR) / (np.sqrt(rhoL) + np.sqrt(rhoR))
    c_hat_sq = (cL ** 2 * np.sqrt(rhoL) + cR ** 2 * np.sqrt(rhoR)) / (np.sqrt(rhoL) + np.sqrt(rhoR)) + 0.5 * (
        np.sqrt(rhoL) * np.sqrt(rhoR) / (np.sqrt(rhoL) + np.sqrt(rhoR)) ** 2) * (uR - uL) ** 2
    c_hat = np.sqrt(c_hat_sq)
    SL = np.minimum(uL - cL, u_hat - c_hat)
    SR = np.maximum(uR + cR, u_hat + c_hat)
    S_star = (pR - pL + rhoL * uL * (SL - uL) - rhoR * uR * (SR - uR)) / (rhoL * (SL - uL) - rhoR * (SR - uR))
    UL = _fv.conserved_state_from_primitive(PL, gamma, dims, rv)
    UR = _fv.conserved_state_from_primitive(PR, gamma, dims, rv)
    USL = np.array(UL, copy=True)
    USL[axis] = rhoL * S_star
    USL[rv.pressure_index] = USL[rv.pressure_index] + (S_star - uL) * (rhoL * S_star + pL / (SL - uL))
    USL = USL * (SL - uL) / (SL - S_star)
    USR = np.array(UR, copy=True)
    USR[axis] = rhoR * S_star
    USR[rv.pressure_index] = USR[rv.pressure_index] + (S_star - uR) * (rhoR * S_star + pR / (SR - uR))
    USR = USR * (SR - uR) / (SR - S_star)
    if config.riemann_solver == HLLC_LM:
        Ma_local = np.maximum(np.abs(uL / cL), np.abs(uR / cR))
        phi = np.sin(np.minimum(1, Ma_local / 0.1) * np.pi / 2)
        SLs, SRs = SL * phi, SR * phi
    else:
        SLs, SRs = SL, SR
    diss = 0.5 * (SLs * (USL - UL) + np.abs(S_star) * (USL - USR) + SRs * (USR - UR))
    f_i_to_im1 = 0.5 * FR + np.minimum(diss, 0)
    f_im1 = 0.5 * FL + np.maximum(diss, 0)
    if config.self_gravity_version == RIEMANN_SPLIT_UNSTABLE:
        f_i_to_im1 = np.where(SR <= 0, FR / 2, f_i_to_im1)
        f_i_to_im1 = np.where(SL >= 0, FL / 2, f_i_to_im1)
        f_im1 = np.where(SL >= 0, FL / 2, f_im1)
        f_im1 = np.where(SR <= 0, FR / 2, f_im1)
    return f_i_to_im1, f_im1


def source_term_along_axis(phi, P, dx, rv, dt, gamma, config, axis):
    """_self_gravity.py:68-337 (`axis` 1-based; `phi` without the variable axis)."""
    rho = P[rv.density_index]
    v_axis = P[axis]
    acc = -_stencil_diff(phi, 1, -1, axis - 1) / (2 * dx)
    src = np.zeros_like(P)
    src[axis] = rho * acc
    version = config.self_gravity_version
    if version == SIMPLE_SOURCE_TERM:
        src[rv.pressure_index] = rho * v_axis * acc
        return src
    PL, PR = _interface_states(P, dt, gamma, config, rv, axis)
    if version in (RIEMANN_SPLIT, RIEMANN_SPLIT_UNSTABLE):
        f_i_to_im1, f_im1 = _riemann_split_fluxes(PL, PR, gamma, config, rv, axis)
        f_i_to_ip1 = np.roll(f_im1, -1, axis)
    elif version == DONOR_ACCOUNTING:
        F = _fv.riemann_solver(PL, PR, P, gamma, config, rv, axis)
        f_i_to_ip1 = np.maximum(np.roll(F, -1, axis), 0)
        f_i_to_im1 = np.minimum(F, 0)
    elif version == HALF_SPLIT:
        F = _fv.riemann_solver(PL, PR, P, gamma, config, rv, axis)
        f_i_to_ip1 = 0.5 * np.roll(F, -1, axis)
        f_i_to_im1 = 0.5 * F
    else:
        raise ValueError("unknown self-gravity version %d" % version)
    acc_b = -_stencil_diff(phi, 0, -1, axis - 1) / dx
    acc_f = -_stencil_diff(phi, 1, 0, axis - 1) / dx
    f_acc = f_i_to_im1 * acc_b + f_i_to_ip1 * acc_f
    src[rv.pressure_index] = f_acc[0]
    return src


def apply_self_gravity(P, P_old, config, rv, gamma, G, dt):
    """_self_gravity.py:341-390: the potential of the old density, the source
    of every axis, one explicit update in conserved variables."""
    dims = config.dimensionality
    rho = P_old[rv.density_index]
    phi = gravitational_potential(rho, config.grid_spacing, config, G)
    src = np.zeros_like(P)
    for i in range(dims):
        src = src + source_term_along_axis(phi, P_old, config.grid_spacing, rv, dt, gamma, config, i + 1)
    U = _fv.conserved_state_from_primitive(P, gamma, dims, rv)
    U = U + dt * src
    P = _fv.primitive_state_from_conserved(U, gamma, dims, rv)
    if config.boundary_handling == GHOST_CELLS:
        P = _fv.boundary_handler(P, config)
    return P


def gravitational_energy(P_unpadded, config, rv, G):
    """total_quantities.py:90-104 (Cartesian)."""
    rho = P_unpadded[rv.density_index]
    phi = gravitational_potential(rho, config.grid_spacing, config, G)
    e = 0.5 * rho * phi
    if config.dimensionality == 1:
        return float(np.sum(e * config.grid_spacing))
    return float(np.sum(e * config.grid_spacing ** config.dimensionality))
