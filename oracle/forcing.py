"""Oracle: turbulent forcing and the FD stellar-wind source (test infrastructure only).

Nothing in the product imports this module; it is the checker for the CUDA
forcing and wind kernels.  It restates astronomix 0.5.1's

* ``_physics_modules/_turbulent_forcing/_turbulent_forcing.py:15-128``
  (``_create_forcing_field``: a k^6 exp(-8k/k_p) spectrum of complex Gaussian
  noise per velocity component, the compressive part projected out, the real
  part of the inverse FFT; ``_apply_forcing``: the amplitude that injects
  ``energy_injection_rate * dt`` of kinetic energy, added to the velocities),
* ``_physics_modules/_stellar_wind/stellar_wind.py:485-584``
  (``_wind_ei3D_source``: the tapered thermal-energy injection source of the
  FD right-hand side).

Random numbers: the reference draws its noise from ``jax.random`` (threefry,
key 42, split every step); that stream cannot be reproduced without JAX.
Both this oracle and the CUDA kernels draw it from Philox4x32-10 (Salmon,
Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11)
keyed by the seed, counter (mode, component, step, 0), two uniforms per
complex draw turned into a normal pair by Box-Muller.  The forcing's
spectrum, projection, normalisation and amplitude equation are the
reference's; its random stream is not.
"""

import numpy as np

_M0 = np.uint64(0xD2511F53)
_M1 = np.uint64(0xCD9E8D57)
_W0 = np.uint32(0x9E3779B9)
_W1 = np.uint32(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Philox4x32 with 10 rounds on arrays of uint32 counters; returns 4 uint32 arrays."""
    c0, c1, c2, c3 = (np.asarray(x, dtype=np.uint32) for x in (c0, c1, c2, c3))
    k0 = np.asarray(k0, dtype=np.uint32)
    k1 = np.asarray(k1, dtype=np.uint32)
    for r in range(10):
        if r:
            k0 = ((k0.astype(np.uint64) + np.uint64(_W0)) & _MASK).astype(np.uint32)
            k1 = ((k1.astype(np.uint64) + np.uint64(_W1)) & _MASK).astype(np.uint32)
        p0 = _M0 * c0.astype(np.uint64)
        p1 = _M1 * c2.astype(np.uint64)
        hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), (p0 & _MASK).astype(np.uint32)
        hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), (p1 & _MASK).astype(np.uint32)
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return c0, c1, c2, c3


def gaussian_noise(seed, step, n):
    """(re, im) normal draws of shape (3, n, n, n) for one forcing step."""
    m = np.arange(n ** 3, dtype=np.uint64)
    re = np.empty((3, n ** 3))
    im = np.empty((3, n ** 3))
    k0 = np.uint32(seed & 0xFFFFFFFF)
    k1 = np.uint32((seed >> 32) & 0xFFFFFFFF)
    for comp in range(3):
        x0, x1, _, _ = philox4x32_10(m.astype(np.uint32), np.uint32(comp), np.uint32(step & 0xFFFFFFFF),
                                     np.uint32((step >> 32) & 0xFFFFFFFF), k0, k1)
        u1 = (x0.astype(np.float64) + 1.0) * 2.0 ** -32
        u2 = x1.astype(np.float64) * 2.0 ** -32
        rr = np.sqrt(-2.0 * np.log(u1))
        th = 2.0 * np.pi * u2
        re[comp] = rr * np.cos(th)
        im[comp] = rr * np.sin(th)
    return re.reshape(3, n, n, n), im.reshape(3, n, n, n)


def create_forcing_field(seed, step, n, box_size):
    """_turbulent_forcing.py:15-70 with the Philox noise above (FP64)."""
    kx = 2.0 * np.pi * np.fft.fftfreq(n, d=box_size / n)
    kx3 = kx.reshape(n, 1, 1)
    ky3 = kx.reshape(1, n, 1)
    kz3 = kx.reshape(1, 1, n)
    k2 = kx3 ** 2 + ky3 ** 2 + kz3 ** 2
    kk = np.sqrt(k2)
    kpk = 4.0 * np.pi / box_size
    Pk = kk ** 6 * np.exp(-8.0 * kk / kpk)
    re, im = gaussian_noise(seed, step, n)
    noise = re + 1j * im
    cw = [np.sqrt(Pk) * noise[c] for c in range(3)]
    for c in range(3):
        cw[c][0, 0, 0] = 0.0
    k2s = np.where(k2 == 0.0, 1.0, k2)
    div_k = (kx3 * cw[0] + ky3 * cw[1] + kz3 * cw[2]) / k2s
    div_k[0, 0, 0] = 0.0
    cw = [cw[0] - kx3 * div_k, cw[1] - ky3 * div_k, cw[2] - kz3 * div_k]
    return [np.real(np.fft.ifftn(c)) for c in cw]


def forcing_amplitude(P, w, dt, energy_injection_rate, dx, rv):
    """_turbulent_forcing.py:72-110: the amplitude that injects Edot dt (per volume dV)."""
    rho = P[rv.density_index]
    v = [P[rv.velocity_index.x], P[rv.velocity_index.y], P[rv.velocity_index.z]]
    dV = dx ** 3
    a = 0.5 * np.sum(rho * (w[0] ** 2 + w[1] ** 2 + w[2] ** 2))
    b = np.sum(rho * v[0] * w[0] + rho * v[1] * w[1] + rho * v[2] * w[2])
    c = -energy_injection_rate * dt / dV
    disc = b ** 2 - 4.0 * a * c
    if disc >= 0 and abs(a) > 1e-10:
        return (-b + np.sqrt(disc)) / (2.0 * a)
    return 0.0


def apply_forcing(P, dt, step, config, params, rv, seed=42):
    """_turbulent_forcing.py:72-128: velocities += amp * w."""
    n = config.num_cells
    w = create_forcing_field(seed, step, n, config.box_size)
    amp = forcing_amplitude(P.astype(np.float64), w, float(dt),
                            params.turbulent_forcing_params.energy_injection_rate, config.grid_spacing, rv)
    P = np.array(P, copy=True)
    for c, idx in enumerate((rv.velocity_index.x, rv.velocity_index.y, rv.velocity_index.z)):
        P[idx] = P[idx] + (amp * w[c]).astype(P.dtype)
    return P


def cell_radius(n, dx, box_size):
    """helper_data.r of get_helper_data (simulation_helper_data.py:49-160):
    distance of every cell centre from the box centre."""
    x = np.linspace(dx / 2, box_size + dx / 2, n, endpoint=False)
    gc = np.moveaxis(np.array(np.meshgrid(x, x, x)), 0, -1)
    return np.linalg.norm(gc - np.zeros(3) - box_size / 2, axis=-1)


def wind_ei3d_source(q, dt, mdot, vinf, r, dx, num_injection_cells):
    """stellar_wind.py:485-584: the EI source of conserved variables over dt
    (rows rho, m_x, m_y, m_z, E); dt is k2 * dt of the SSPRK stage."""
    src = np.zeros_like(q)
    r_inj = num_injection_cells * dx
    r_1 = 1.3 * r_inj
    mask = np.where(r <= r_inj, 1.0, np.where((r > r_inj) & (r <= r_1), (r_1 - r) / (r_1 - r_inj), 0.0))
    V = np.sum(mask) * dx ** 3
    drho_dt = mdot / V
    src[0] = drho_dt * mask * dt
    dE = 0.5 * vinf ** 2 * mdot / V * dt
    with np.errstate(invalid="ignore", divide="ignore"):
        f = np.sqrt(1 + drho_dt * dt * mask / q[0]) - 1.0
    f = np.where(r <= r_1, f, 0.0)
    for k in (1, 2, 3):
        src[k] = q[k] * f
    src[4] = dE * mask
    return src
