"""Exact solution of the 1D Euler Riemann problem (test infrastructure).

The reference validates its Sod shock tube against ExactPack's exact Riemann
solver (tests/hydro_tests/shock_tube.py:109-134); ExactPack is not available
here, so this module solves the same problem from the textbook mathematics:
the star-region pressure is the root of f_L(p) + f_R(p) + (u_R - u_L) = 0
(Newton iteration), with shock (Rankine-Hugoniot) or rarefaction (isentropic)
branches on each side, and the solution is sampled at x / t.
"""

import numpy as np


def _f_and_df(p, rho_k, p_k, gamma):
    c_k = np.sqrt(gamma * p_k / rho_k)
    if p > p_k:  # shock
        A = 2.0 / ((gamma + 1.0) * rho_k)
        B = (gamma - 1.0) / (gamma + 1.0) * p_k
        sq = np.sqrt(A / (p + B))
        f = (p - p_k) * sq
        df = sq * (1.0 - 0.5 * (p - p_k) / (B + p))
    else:  # rarefaction
        f = 2.0 * c_k / (gamma - 1.0) * ((p / p_k) ** ((gamma - 1.0) / (2.0 * gamma)) - 1.0)
        df = 1.0 / (rho_k * c_k) * (p / p_k) ** (-(gamma + 1.0) / (2.0 * gamma))
    return f, df


def star_state(rho_l, u_l, p_l, rho_r, u_r, p_r, gamma, tol=1e-14, max_iter=100):
    """Pressure and velocity of the star region."""
    p = max(0.5 * (p_l + p_r), 1e-12)
    for _ in range(max_iter):
        fl, dfl = _f_and_df(p, rho_l, p_l, gamma)
        fr, dfr = _f_and_df(p, rho_r, p_r, gamma)
        p_new = p - (fl + fr + u_r - u_l) / (dfl + dfr)
        p_new = max(p_new, 1e-14)
        if abs(p_new - p) < tol * 0.5 * (p_new + p):
            p = p_new
            break
        p = p_new
    fl, _ = _f_and_df(p, rho_l, p_l, gamma)
    fr, _ = _f_and_df(p, rho_r, p_r, gamma)
    u = 0.5 * (u_l + u_r) + 0.5 * (fr - fl)
    return p, u


def sample(x, t, x0, left, right, gamma):
    """rho, u, p of the exact solution at positions x (array) and time t > 0."""
    rho_l, u_l, p_l = left
    rho_r, u_r, p_r = right
    ps, us = star_state(rho_l, u_l, p_l, rho_r, u_r, p_r, gamma)
    g = gamma
    c_l = np.sqrt(g * p_l / rho_l)
    c_r = np.sqrt(g * p_r / rho_r)
    xi = (np.asarray(x, dtype=np.float64) - x0) / t
    rho = np.empty_like(xi)
    u = np.empty_like(xi)
    p = np.empty_like(xi)
    for i, s in enumerate(xi):
        if s <= us:  # left of the contact
            if ps > p_l:  # left shock
                rho_s = rho_l * ((ps / p_l + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / p_l + 1))
                S = u_l - c_l * np.sqrt((g + 1) / (2 * g) * ps / p_l + (g - 1) / (2 * g))
                rho[i], u[i], p[i] = (rho_l, u_l, p_l) if s <= S else (rho_s, us, ps)
            else:  # left rarefaction
                rho_s = rho_l * (ps / p_l) ** (1 / g)
                c_s = c_l * (ps / p_l) ** ((g - 1) / (2 * g))
                head, tail = u_l - c_l, us - c_s
                if s <= head:
                    rho[i], u[i], p[i] = rho_l, u_l, p_l
                elif s >= tail:
                    rho[i], u[i], p[i] = rho_s, us, ps
                else:
                    fac = 2 / (g + 1) + (g - 1) / ((g + 1) * c_l) * (u_l - s)
                    rho[i] = rho_l * fac ** (2 / (g - 1))
                    u[i] = 2 / (g + 1) * (c_l + (g - 1) / 2 * u_l + s)
                    p[i] = p_l * fac ** (2 * g / (g - 1))
        else:  # right of the contact
            if ps > p_r:  # right shock
                rho_s = rho_r * ((ps / p_r + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / p_r + 1))
                S = u_r + c_r * np.sqrt((g + 1) / (2 * g) * ps / p_r + (g - 1) / (2 * g))
                rho[i], u[i], p[i] = (rho_r, u_r, p_r) if s >= S else (rho_s, us, ps)
            else:  # right rarefaction
                rho_s = rho_r * (ps / p_r) ** (1 / g)
                c_s = c_r * (ps / p_r) ** ((g - 1) / (2 * g))
                head, tail = u_r + c_r, us + c_s
                if s >= head:
                    rho[i], u[i], p[i] = rho_r, u_r, p_r
                elif s <= tail:
                    rho[i], u[i], p[i] = rho_s, us, ps
                else:
                    fac = 2 / (g + 1) - (g - 1) / ((g + 1) * c_r) * (u_r - s)
                    rho[i] = rho_r * fac ** (2 / (g - 1))
                    u[i] = 2 / (g + 1) * (-c_r + (g - 1) / 2 * u_r + s)
                    p[i] = p_r * fac ** (2 * g / (g - 1))
    return rho, u, p
