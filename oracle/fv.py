"""Oracle: CPU restatement of the reference's finite-volume path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; it is
the checker that the CUDA kernels are compared against.  Every function
restates the reference JAX code operation for operation (same operand order,
same roll/ghost-cell semantics, same where-branches), on padded arrays exactly
as the reference holds them.  Citations are file:line in leo1200/astronomix
0.5.1.

Arrays: ``state[var, x(, y(, z))]``; the spatial axis ``a`` (1-based, like the
reference's ``axis`` argument) is array axis ``a``.
"""

from astronomix_gb300.option_classes import (
    GHOST_CELLS, OPEN_BOUNDARY, REFLECTIVE_BOUNDARY, PERIODIC_BOUNDARY,
    MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE, VAN_ALBADA, VAN_ALBADA_PP,
    HLL, HLLC, HLLC_LM, LAX_FRIEDRICHS, HYBRID_HLLC, AM_HLLC, UNSPLIT, RK2_SSP, MUSCL,
    IMPLICIT_MIDPOINT, IMPLICIT_EULER, SINGLE_PRECISION, DOUBLE_PRECISION,
)
from ._xp import xp


def _vel_rows(rv, dims):
    if dims == 1:
        return [rv.velocity_index]
    v = rv.velocity_index
    return [v.x, v.y, v.z][:dims]


# ----------------------------------------------------------------- padding

def pad(state, dims):
    """Edge-pad 2 cells per side (time_stepping/_utils.py:65-75)."""
    return xp.pad_edge(state, 2, dims)


def unpad(state, dims, g=2):
    """Slice the ghost cells off (time_stepping/_utils.py:19-60)."""
    sl = (slice(None),) + (slice(g, -g),) * dims
    return state[sl]


# ---------------------------------------------------------- boundaries

def _set_along_axis(s, axis, set_index, get_index):
    # _geometry/boundaries.py:23-39
    # in place: boundary_handler owns a private copy of the state
    idx_set = (slice(None),) * axis + (set_index,)
    idx_get = (slice(None),) * axis + (get_index,)
    s[idx_set] = s[idx_get]
    return s


def _set_var_along_axis(s, axis, set_index, get_index, var_index, factor):
    # _geometry/boundaries.py:46-69.  A var_index beyond the array's rows (the
    # 3D z wall of the magnetic update's 3-vectors: var_index 3) is an update
    # that JAX drops (.at[] scatters skip out-of-range indices): no change.
    if var_index >= s.shape[0]:
        return s
    idx_set = (var_index,) + (slice(None),) * (axis - 1) + (set_index,)
    idx_get = (var_index,) + (slice(None),) * (axis - 1) + (get_index,)
    s[idx_set] = factor * s[idx_get]
    return s


def _open_left(s, g, axis):
    for set_index in range(g):
        s = _set_along_axis(s, axis, set_index, g)
    return s


def _open_right(s, g, axis):
    for set_index in range(-g, 0):
        s = _set_along_axis(s, axis, set_index, -g - 1)
    return s


def _periodic(s, g, axis):
    # _geometry/boundaries.py:298-319
    for i in range(g):
        s = _set_along_axis(s, axis, i, i - 2 * g)
        s = _set_along_axis(s, axis, -i - 1, 2 * g - i - 1)
    return s


def _reflective_left(s, g, axis):
    # _geometry/boundaries.py:324-337
    for i in range(g):
        get_index = i + g
        set_index = g - i - 1
        s = _set_along_axis(s, axis, set_index, get_index)
        s = _set_var_along_axis(s, axis, set_index, get_index, axis, -1.0)
    return s


def _reflective_right(s, g, axis):
    # _geometry/boundaries.py:342-355
    for i in range(g):
        get_index = -i - g - 1
        set_index = -g + i
        s = _set_along_axis(s, axis, set_index, get_index)
        s = _set_var_along_axis(s, axis, set_index, get_index, axis, -1.0)
    return s


def _reflective_left_1d(s):
    # _geometry/boundaries.py:360-370
    s[:, 0] = s[:, 2]
    s[1, 0] = -s[1, 2]
    s[:, 1] = s[:, 2]
    s[1, 1] = -s[1, 2]
    return s


def _reflective_right_1d(s):
    # _geometry/boundaries.py:375-385
    s[:, -1] = s[:, -3]
    s[1, -1] = -s[1, -3]
    s[:, -2] = s[:, -3]
    s[1, -2] = -s[1, -3]
    return s


def boundary_handler(s, config):
    """Ghost-cell fill (_geometry/boundaries.py:74-265).

    Order of application is the reference's: open (x, y, z), reflective,
    periodic per axis.
    """
    g = config.num_ghost_cells
    bs = config.boundary_settings
    d = config.dimensionality
    s = xp.copy(s)
    if d == 1:
        if bs.left_boundary == OPEN_BOUNDARY:
            s = _open_left(s, g, 1)
        elif bs.left_boundary == REFLECTIVE_BOUNDARY:
            s = _reflective_left_1d(s)
        if bs.right_boundary == OPEN_BOUNDARY:
            s = _open_right(s, g, 1)
        elif bs.right_boundary == REFLECTIVE_BOUNDARY:
            s = _reflective_right_1d(s)
        if bs.left_boundary == PERIODIC_BOUNDARY and bs.right_boundary == PERIODIC_BOUNDARY:
            s = _periodic(s, g, 1)
        return s
    axes = [bs.x, bs.y, bs.z][:d]
    for a, b in enumerate(axes, start=1):
        if b.left_boundary == OPEN_BOUNDARY:
            s = _open_left(s, g, a)
        if b.right_boundary == OPEN_BOUNDARY:
            s = _open_right(s, g, a)
    for a, b in enumerate(axes, start=1):
        if b.left_boundary == REFLECTIVE_BOUNDARY:
            s = _reflective_left(s, g, a)
        if b.right_boundary == REFLECTIVE_BOUNDARY:
            s = _reflective_right(s, g, a)
    for a, b in enumerate(axes, start=1):
        if b.left_boundary == PERIODIC_BOUNDARY and b.right_boundary == PERIODIC_BOUNDARY:
            s = _periodic(s, g, a)
    return s


# ------------------------------------------------------- fluid equations

def get_absolute_velocity(P, dims, rv):
    # _fluid_equations/_equations.py:165-199
    if dims == 1:
        return xp.abs(P[rv.velocity_index])
    v = rv.velocity_index
    if dims == 2:
        return xp.sqrt(P[v.x] ** 2 + P[v.y] ** 2)
    return xp.sqrt(P[v.x] ** 2 + P[v.y] ** 2 + P[v.z] ** 2 + 1e-20)


def total_energy_from_primitives(rho, u, p, gamma):
    # _fluid_equations/_equations.py:253-266
    return p / (gamma - 1) + 0.5 * rho * u ** 2


def pressure_from_energy(E, rho, u, gamma):
    # _fluid_equations/_equations.py:203-248
    e = E / rho - 0.5 * u ** 2
    return (gamma - 1) * rho * e


def speed_of_sound(rho, p, gamma):
    # _fluid_equations/_equations.py:269-280
    return xp.sqrt(gamma * p / rho)


def primitive_state_from_conserved(U, gamma, dims, rv):
    # _fluid_equations/_equations.py:24-94
    rho = U[rv.density_index]
    E = U[rv.pressure_index]
    P = xp.copy(U)
    if dims == 1:
        u = U[rv.velocity_index] / rho
        P[rv.pressure_index] = pressure_from_energy(E, rho, u, gamma)
        P[rv.velocity_index] = u
        return P
    v = rv.velocity_index
    ux = U[v.x] / rho
    uy = U[v.y] / rho
    if dims == 2:
        u = xp.sqrt(ux ** 2 + uy ** 2 + 1e-20)
    else:
        uz = U[v.z] / rho
        u = xp.sqrt(ux ** 2 + uy ** 2 + uz ** 2 + 1e-20)
    P[rv.pressure_index] = pressure_from_energy(E, rho, u, gamma)
    P[v.x] = ux
    P[v.y] = uy
    if dims == 3:
        P[v.z] = uz
    return P


def conserved_state_from_primitive(P, gamma, dims, rv):
    # _fluid_equations/_equations.py:104-156
    rho = P[rv.density_index]
    u = get_absolute_velocity(P, dims, rv)
    p = P[rv.pressure_index]
    U = xp.copy(P)
    U[rv.pressure_index] = total_energy_from_primitives(rho, u, p, gamma)
    for vi in _vel_rows(rv, dims):
        U[vi] = rho * P[vi]
    return U


def euler_flux(P, gamma, dims, rv, d):
    # _fluid_equations/_fluxes.py:25-93 ; d = flux direction index (= axis)
    rho = P[rv.density_index]
    p = P[rv.pressure_index]
    utotal = get_absolute_velocity(P, dims, rv)
    E = total_energy_from_primitives(rho, utotal, p, gamma)
    F = xp.copy(P)
    F[rv.pressure_index] = F[rv.pressure_index] + E
    for vi in _vel_rows(rv, dims):
        F[vi] = P[vi] * rho
    F = P[d] * F
    F[d] = F[d] + p
    return F


# ------------------------------------------------------ reconstruction

def _minmod(a, b):
    # _finite_volume/_state_evolution/limiters.py:14-15
    return 0.5 * (xp.sign(a) + xp.sign(b)) * xp.minimum(xp.abs(a), xp.abs(b))


def _minmod3(a, b, c):
    same = (xp.sign(a) == xp.sign(b)) & (xp.sign(b) == xp.sign(c))
    return xp.where(same, xp.sign(a) * xp.minimum(xp.abs(a), xp.minimum(xp.abs(b), xp.abs(c))), 0.0)


def _double_minmod(a, b):
    # limiters.py:28-32
    return xp.where(a * b > 0, _minmod3((a + b) / 2, 2 * a, 2 * b), 0.0)


def _maxmod(a, b):
    return 0.5 * (xp.sign(a) + xp.sign(b)) * xp.maximum(xp.abs(a), xp.abs(b))


def _superbee(a, b):
    # limiters.py:40-44
    return xp.where(a * b > 0, _minmod(_maxmod(a, b), _minmod(2 * a, 2 * b)), 0.0)


def _van_albada(bd, fd, dx):
    # limiters.py:48-64
    eps = 3 * dx
    return ((fd ** 2 + eps) * bd + (bd ** 2 + eps) * fd) / (fd ** 2 + bd ** 2 + 2 * eps)


def limited_gradients(P, config, axis):
    """_finite_volume/_state_evolution/limited_gradients.py:22-88 (Cartesian)."""
    dx = config.grid_spacing
    bd = (P - xp.roll(P, 1, axis)) / dx
    fd = (xp.roll(P, -1, axis) - P) / dx
    lim = config.limiter
    if lim == MINMOD:
        return _minmod(bd, fd)
    if lim == SUPERBEE:
        return _superbee(bd, fd)
    if lim == DOUBLE_MINMOD:
        return _double_minmod(bd, fd)
    if lim in (VAN_ALBADA, VAN_ALBADA_PP):
        return _van_albada(bd, fd, dx)
    if lim == OSHER:
        eps = 1e-11
        g = xp.where(xp.abs(bd) > eps, fd / (bd + eps), xp.zeros_like(bd))
        return xp.maximum(0, xp.minimum(1.3, g)) * bd
    raise NotImplementedError("limiter %d is not part of the accelerated path" % lim)


def reconstruct_unsplit_single(P, config, axis):
    """reconstruction.py:399-431: returns (p_left_interface, p_right_interface)."""
    g = limited_gradients(P, config, axis)
    diff = g * config.grid_spacing / 2
    left_center = P - diff
    right_center = P + diff
    return xp.roll(right_center, 1, axis), left_center


def reconstruct_split(P, dt, gamma, config, rv, axis):
    """reconstruction.py:40-129 (Cartesian): limited gradients, the MUSCL-Hancock
    half-step predictor P - dt/2 A_W g with the reference's A_W (u on the
    diagonal, A[rho, axis] = rho, A[p, 1] = rho c^2 -- column 1 whatever the
    axis, as the reference sets it -- and A[axis, p] = 1 / rho; the einsum's
    sum over a taken in increasing a), and the interface states."""
    if config.time_integrator != MUSCL:
        raise ValueError("Time integrator %d not supported for split reconstruction. Only MUSCL is supported."
                         % config.time_integrator)
    rho = P[rv.density_index]
    p = P[rv.pressure_index]
    u = P[axis]
    g = limited_gradients(P, config, axis)
    c = speed_of_sound(rho, p, gamma)
    nv = P.shape[0]
    pi = rv.pressure_index
    proj = xp.zeros_like(P)
    for b in range(nv):
        coef = {b: u}
        if b == rv.density_index:
            coef[axis] = rho
        if b == pi:
            coef[1] = rho * c ** 2
        if b == axis:
            coef[pi] = 1 / rho
        acc = None
        for a_ in sorted(coef):
            term = coef[a_] * g[a_]
            acc = term if acc is None else acc + term
        proj[b] = acc
    predictors = P - dt / 2 * proj
    dist = config.grid_spacing / 2
    left = predictors - dist * g
    right = predictors + dist * g
    return xp.roll(right, 1, axis), left


def reconstruct_unsplit_pp(P, gamma, config, rv, C_cfl):
    """reconstruction.py:134-394, the VAN_ALBADA_PP branch (2D / 3D): van
    Albada differences along every axis, rescaled per cell for positivity.
    C_k = alpha_k / sum(alpha) from the global maxima of |u_k| + c; the
    density and pressure differences of axis k are limited by alpha_k,
    kappa_k; the velocity differences by one beta per cell, whose A1 pairs
    the axis-j factors with velocity component j (the reference's
    broadcasting of C * alpha * d_rho against the (axis, component) array of
    velocity differences).  Returns [(p_left_interface, p_right_interface)]
    per axis."""
    dims = config.dimensionality
    if dims < 2:
        raise NotImplementedError("VAN_ALBADA_PP in 1D sums over the whole grid in the reference; "
                                  "not part of the accelerated path")
    eps = 1e-14
    d = [limited_gradients(P, config, axis) * config.grid_spacing / 2 for axis in range(1, dims + 1)]
    ri, pi = rv.density_index, rv.pressure_index
    rho = P[ri]
    p = P[pi]
    c = speed_of_sound(rho, p, gamma)
    alpha_lax = [xp.amax(xp.abs(P[axis]) + c) for axis in range(1, dims + 1)]
    tot = alpha_lax[0]
    for a_ in alpha_lax[1:]:
        tot = tot + a_
    C = [a_ / tot for a_ in alpha_lax]
    q = (2 / C_cfl) if config.mhd else (1 / C_cfl)

    def limit(x, ref):
        prot = xp.where(xp.abs(x) > eps, x, eps)
        return xp.where(xp.abs(x) > eps, xp.minimum(ref / (xp.abs(prot) * (1 + eps)), 1), 1)

    alpha_d = [limit(d[k][ri], rho) for k in range(dims)]
    kappa_p = [limit(d[k][pi], p) for k in range(dims)]
    A1 = None
    for j in range(dims):
        X = C[j] * alpha_d[j] * d[j][ri]
        S = None
        for k in range(dims):
            term = X * d[k][1 + j]
            S = term if S is None else S + term
        A1 = S ** 2 if A1 is None else A1 + S ** 2
    A2 = None
    vsum = None
    for k in range(dims):
        sq_ = None
        for j in range(dims):
            t_ = d[k][1 + j] ** 2
            sq_ = t_ if sq_ is None else sq_ + t_
        term = C[k] * sq_
        A2 = term if A2 is None else A2 + term
        vsum = sq_ if vsum is None else vsum + sq_
    A1 = xp.where(vsum > eps, A1, eps)
    A2 = xp.where(vsum > eps, A2, eps)
    beta = xp.where(vsum > eps,
                    xp.minimum(xp.sqrt(((q - 2) ** 2 * rho * p) / ((gamma - 1) * (2 * A1 + (q - 2) * rho ** 2 * A2))),
                               1), 1)
    out = []
    for k in range(dims):
        dk = xp.copy(d[k])
        dk[ri] = d[k][ri] * alpha_d[k]
        dk[pi] = d[k][pi] * kappa_p[k]
        for j in range(dims):
            dk[1 + j] = d[k][1 + j] * beta
        left_center = P - dk
        right_center = P + dk
        out.append((xp.roll(right_center, 1, k + 1), left_center))
    return out


# ------------------------------------------------------ Riemann solvers

def hll(PL, PR, gamma, dims, rv, d):
    """_finite_volume/_riemann_solver/hll.py:36-109."""
    rhoL, uL, pL = PL[rv.density_index], PL[d], PL[rv.pressure_index]
    rhoR, uR, pR = PR[rv.density_index], PR[d], PR[rv.pressure_index]
    cL = speed_of_sound(rhoL, pL, gamma)
    cR = speed_of_sound(rhoR, pR, gamma)
    FL = euler_flux(PL, gamma, dims, rv, d)
    FR = euler_flux(PR, gamma, dims, rv, d)
    SR = xp.maximum(xp.maximum(uL + cL, uR + cR), 0)
    SL = xp.minimum(xp.minimum(uL - cL, uR - cR), 0)
    UL = conserved_state_from_primitive(PL, gamma, dims, rv)
    UR = conserved_state_from_primitive(PR, gamma, dims, rv)
    return (SR * FL - SL * FR + SL * SR * (UR - UL)) / (SR - SL)


def hllc(PL, PR, gamma, dims, rv, d, lm=False, lmdc=False):
    """_finite_volume/_riemann_solver/hll.py:123-261 (HLLC and HLLC-LM;
    `lmdc`: the low-Mach dissipation control of the velocity rows, :230-254)."""
    rhoL, uL, pL = PL[rv.density_index], PL[d], PL[rv.pressure_index]
    rhoR, uR, pR = PR[rv.density_index], PR[d], PR[rv.pressure_index]
    cL = speed_of_sound(rhoL, pL, gamma)
    cR = speed_of_sound(rhoR, pR, gamma)
    FL = euler_flux(PL, gamma, dims, rv, d)
    FR = euler_flux(PR, gamma, dims, rv, d)
    u_hat = (xp.sqrt(rhoL) * uL + xp.sqrt(rhoR) * uR) / (xp.sqrt(rhoL) + xp.sqrt(rhoR))
    c_hat_sq = (cL ** 2 * xp.sqrt(rhoL) + cR ** 2 * xp.sqrt(rhoR)) / (
        xp.sqrt(rhoL) + xp.sqrt(rhoR)
    ) + 0.5 * (
        xp.sqrt(rhoL) * xp.sqrt(rhoR) / (xp.sqrt(rhoL) + xp.sqrt(rhoR)) ** 2
    ) * (uR - uL) ** 2
    c_hat = xp.sqrt(c_hat_sq)
    SL = xp.minimum(uL - cL, u_hat - c_hat)
    SR = xp.maximum(uR + cR, u_hat + c_hat)
    S_star = (pR - pL + rhoL * uL * (SL - uL) - rhoR * uR * (SR - uR)) / (
        rhoL * (SL - uL) - rhoR * (SR - uR)
    )
    UL = conserved_state_from_primitive(PL, gamma, dims, rv)
    UR = conserved_state_from_primitive(PR, gamma, dims, rv)
    USL = xp.copy(UL)
    USL[d] = rhoL * S_star
    USL[rv.pressure_index] = USL[rv.pressure_index] + (S_star - uL) * (rhoL * S_star + pL / (SL - uL))
    USL = USL * (SL - uL) / (SL - S_star)
    USR = xp.copy(UR)
    USR[d] = rhoR * S_star
    USR[rv.pressure_index] = USR[rv.pressure_index] + (S_star - uR) * (rhoR * S_star + pR / (SR - uR))
    USR = USR * (SR - uR) / (SR - S_star)
    if lm:
        Ma_local = xp.maximum(xp.abs(uL / cL), xp.abs(uR / cR))
        phi = xp.sin(xp.minimum(1, Ma_local / 0.1) * 3.141592653589793 / 2)
        SLs = SL * phi
        SRs = SR * phi
    else:
        SLs, SRs = SL, SR
    diss = 0.5 * (SLs * (USL - UL) + xp.abs(S_star) * (USL - USR) + SRs * (USR - UR))
    if lmdc:
        Ma = xp.maximum(xp.abs(get_absolute_velocity(PL, dims, rv) / cL),
                        xp.abs(get_absolute_velocity(PR, dims, rv) / cR))
        f = xp.minimum(1, Ma)
        v0 = rv.velocity_index if dims == 1 else rv.velocity_index.x
        diss = xp.copy(diss)
        diss[v0:v0 + dims] = f * diss[v0:v0 + dims]
    F_star = 0.5 * (FL + FR) + diss
    F = xp.where(SL >= 0, FL, F_star)
    F = xp.where(SR <= 0, FR, F)
    return F


def am_hllc(PL, PR, P, gamma, config, rv, d):
    """_finite_volume/_riemann_solver/hll.py:268-326: HLLC-LM where the cell
    right of the interface is compressed (div v < -0.05 c / dx, central
    differences of the stage state), HLLC elsewhere; AM_HLLC with the
    low-Mach dissipation control, HYBRID_HLLC without."""
    dims = config.dimensionality
    dx = config.grid_spacing
    a = speed_of_sound(P[rv.density_index], P[rv.pressure_index], gamma)
    div_v = 0
    for i in range(dims):
        # _stencil_add(v_i, indices=(1, -1), factors=(1, -1), axis=i) / (2 dx)
        div_v = div_v + (0 + 1.0 * xp.roll(P[i + 1], -1, i) + (-1.0) * xp.roll(P[i + 1], 1, i)) / (2 * dx)
    g = xp.where(div_v < -0.05 * a / dx, 1, 0)
    lmdc = config.riemann_solver == AM_HLLC
    F_hllc = hllc(PL, PR, gamma, dims, rv, d, lm=False, lmdc=lmdc)
    F_lm = hllc(PL, PR, gamma, dims, rv, d, lm=True, lmdc=lmdc)
    return g * F_lm + (1 - g) * F_hllc


def lax_friedrichs(PL, PR, P, gamma, dims, rv, d):
    """_finite_volume/_riemann_solver/_lax_friedrichs.py:21-78 (global alpha)."""
    UL = conserved_state_from_primitive(PL, gamma, dims, rv)
    UR = conserved_state_from_primitive(PR, gamma, dims, rv)
    u = P[d]
    c = speed_of_sound(P[rv.density_index], P[rv.pressure_index], gamma)
    alpha = xp.amax(xp.abs(u) + c)
    FL = euler_flux(PL, gamma, dims, rv, d)
    FR = euler_flux(PR, gamma, dims, rv, d)
    return 0.5 * (FL + FR) - 0.5 * alpha * (UR - UL)


def riemann_solver(PL, PR, P, gamma, config, rv, d):
    """_finite_volume/_riemann_solver/_riemann_solver.py:37-87."""
    rs = config.riemann_solver
    dims = config.dimensionality
    if rs == HLL:
        return hll(PL, PR, gamma, dims, rv, d)
    if rs == HLLC:
        return hllc(PL, PR, gamma, dims, rv, d)
    if rs == HLLC_LM:
        return hllc(PL, PR, gamma, dims, rv, d, lm=True)
    if rs == LAX_FRIEDRICHS:
        return lax_friedrichs(PL, PR, P, gamma, dims, rv, d)
    if rs in (AM_HLLC, HYBRID_HLLC):
        return am_hllc(PL, PR, P, gamma, config, rv, d)
    raise NotImplementedError("Riemann solver %d is not part of the accelerated path" % rs)


# ------------------------------------------------------- hydro stepper

def evolve_gas_unsplit_inner(P, dt, gamma, config, rv, C_cfl=None):
    """_finite_volume/_state_evolution/evolve_state.py:339-414."""
    dims = config.dimensionality
    ghost = config.boundary_handling == GHOST_CELLS
    if ghost:
        P = boundary_handler(P, config)
    U = conserved_state_from_primitive(P, gamma, dims, rv)
    pp = reconstruct_unsplit_pp(P, gamma, config, rv, C_cfl) if config.limiter == VAN_ALBADA_PP else None
    for axis in range(1, dims + 1):
        if ghost:
            P = boundary_handler(P, config)
        if pp is not None:
            PL, PR = pp[axis - 1]
        else:
            PL, PR = reconstruct_unsplit_single(P, config, axis)
        F = riemann_solver(PL, PR, P, gamma, config, rv, axis)
        U = U + 1 / config.grid_spacing * (F - xp.roll(F, -1, axis)) * dt
    P = primitive_state_from_conserved(U, gamma, dims, rv)
    if ghost:
        P = boundary_handler(P, config)
    return P


def evolve_gas_unsplit(P, dt, gamma, config, rv, C_cfl=None):
    """evolve_state.py:419-488 (SSP-RK2 / Heun in conserved variables)."""
    if config.time_integrator != RK2_SSP:
        raise ValueError("Only the RK2 SSP time integrator is supported for the unsplit scheme.")
    dims = config.dimensionality
    P1 = evolve_gas_unsplit_inner(P, dt, gamma, config, rv, C_cfl)
    P2 = evolve_gas_unsplit_inner(P1, dt, gamma, config, rv, C_cfl)
    U0 = conserved_state_from_primitive(P, gamma, dims, rv)
    U2 = conserved_state_from_primitive(P2, gamma, dims, rv)
    U = 0.5 * (U0 + U2)
    return primitive_state_from_conserved(U, gamma, dims, rv)


def evolve_along_axis(P, dt, gamma, config, rv, axis):
    """evolve_state.py:52-160 (Cartesian): one split sweep along `axis`."""
    dims = config.dimensionality
    ghost = config.boundary_handling == GHOST_CELLS
    if ghost:
        P = boundary_handler(P, config)
    U = conserved_state_from_primitive(P, gamma, dims, rv)
    if config.first_order_fallback:
        PL, PR = xp.roll(P, 1, axis), P
    else:
        PL, PR = reconstruct_split(P, dt, gamma, config, rv, axis)
    F = riemann_solver(PL, PR, P, gamma, config, rv, axis)
    U = U + 1 / config.grid_spacing * (F - xp.roll(F, -1, axis)) * dt
    P = primitive_state_from_conserved(U, gamma, dims, rv)
    if ghost:
        P = boundary_handler(P, config)
    return P


def evolve_gas_split(P, dt, gamma, config, rv):
    """evolve_state.py:168-325: Strang splitting of the axis sweeps."""
    dims = config.dimensionality
    if dims == 1:
        return evolve_along_axis(P, dt, gamma, config, rv, 1)
    if dims == 2:
        P = evolve_along_axis(P, dt / 2, gamma, config, rv, 1)
        P = evolve_along_axis(P, dt, gamma, config, rv, 2)
        return evolve_along_axis(P, dt / 2, gamma, config, rv, 1)
    P = evolve_along_axis(P, dt / 2, gamma, config, rv, 1)
    P = evolve_along_axis(P, dt / 2, gamma, config, rv, 2)
    P = evolve_along_axis(P, dt, gamma, config, rv, 3)
    P = evolve_along_axis(P, dt / 2, gamma, config, rv, 2)
    return evolve_along_axis(P, dt / 2, gamma, config, rv, 1)


def evolve_gas(P, dt, gamma, config, rv, C_cfl=None, G=1.0):
    """The gas update of the configured scheme; with self-gravity, followed by
    the source term of the potential of the density it started from
    (evolve_state.py:178-322, 429-487)."""
    P_old = P
    if config.split == UNSPLIT:
        P = evolve_gas_unsplit(P, dt, gamma, config, rv, C_cfl)
    else:
        P = evolve_gas_split(P, dt, gamma, config, rv)
    if getattr(config, "self_gravity", False):
        from .gravity import apply_self_gravity
        P = apply_self_gravity(P, P_old, config, rv, gamma, G, dt)
    return P


# ----------------------------------------------- magnetic sub-step (Pang-Wu)

def cross(a, b):
    # _finite_volume/_magnetic_update/_vector_maths.py:6-11
    r = xp.zeros_like(a)
    r[0] = a[1] * b[2] - a[2] * b[1]
    r[1] = a[2] * b[0] - a[0] * b[2]
    r[2] = a[0] * b[1] - a[1] * b[0]
    return r


def curl2D(f, dx):
    # _vector_maths.py:80-100 (field axes: 0 = x, 1 = y of each component)
    c = xp.zeros_like(f)
    dFz_dy = 0.5 * (xp.roll(f[2], -1, 1) - xp.roll(f[2], 1, 1)) / dx
    c[0] = c[0] + dFz_dy
    dFz_dx = 0.5 * (xp.roll(f[2], -1, 0) - xp.roll(f[2], 1, 0)) / dx
    c[1] = c[1] + (-dFz_dx)
    dFy_dx = 0.5 * (xp.roll(f[1], -1, 0) - xp.roll(f[1], 1, 0)) / dx
    dFx_dy = 0.5 * (xp.roll(f[0], -1, 1) - xp.roll(f[0], 1, 1)) / dx
    c[2] = c[2] + (dFy_dx - dFx_dy)
    return c


def curl3D(f, dx):
    # _vector_maths.py:55-76
    c = xp.zeros_like(f)
    dFz_dy = 0.5 * (xp.roll(f[2], -1, 1) - xp.roll(f[2], 1, 1)) / dx
    dFy_dz = 0.5 * (xp.roll(f[1], -1, 2) - xp.roll(f[1], 1, 2)) / dx
    c[0] = c[0] + (dFz_dy - dFy_dz)
    dFx_dz = 0.5 * (xp.roll(f[0], -1, 2) - xp.roll(f[0], 1, 2)) / dx
    dFz_dx = 0.5 * (xp.roll(f[2], -1, 0) - xp.roll(f[2], 1, 0)) / dx
    c[1] = c[1] + (dFx_dz - dFz_dx)
    dFy_dx = 0.5 * (xp.roll(f[1], -1, 0) - xp.roll(f[1], 1, 0)) / dx
    dFx_dy = 0.5 * (xp.roll(f[0], -1, 1) - xp.roll(f[0], 1, 1)) / dx
    c[2] = c[2] + (dFy_dx - dFx_dy)
    return c


def divergence(f, dx, dims):
    # _vector_maths.py:15-51
    out = None
    for a in range(dims):
        t = (xp.roll(f[a], -1, a) - xp.roll(f[a], 1, a)) / (2 * dx)
        out = t if out is None else out + t
    return out


def _norm0(a):
    return xp.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])


# the fixed point's iteration cap (_magnetic_field_update.py:141); a module
# constant so that a test can lower it to follow a capped GPU run
MAX_FIXED_POINT_ITERATIONS = 1000


def magnetic_update(B, gas, dx, dt, config, rv, return_iterations=False):
    """_finite_volume/_magnetic_update/_magnetic_field_update.py:37-242.

    Returns ``(B_n, gas_state)`` (and the number of fixed-point iterations
    executed after the first explicit evaluation when requested).
    """
    dims = config.dimensionality
    if dims == 2:
        velocity = xp.zeros_like(B)
        velocity[0:2] = gas[rv.velocity_index.x: rv.velocity_index.x + 2]
    elif dims == 3:
        velocity = xp.copy(gas[rv.velocity_index.x: rv.velocity_index.x + 3])
    else:
        raise ValueError("No 1D MHD.")
    density = gas[rv.density_index]
    curl = curl2D if dims == 2 else curl3D

    def phi(v, b):
        E = cross(b, v)
        phi1 = curl(E, dx)
        phi2 = cross(b, curl(b, dx)) / density
        return phi1, phi2

    ghost = config.boundary_handling == GHOST_CELLS
    if ghost:
        B = boundary_handler(B, config)
        velocity = boundary_handler(velocity, config)
    B0, v0 = B, velocity
    phiA, phiB = phi((v0 + velocity) / 2, (B0 + B) / 2)
    B1 = B - dt * phiA
    v1 = velocity - dt * phiB
    if ghost:
        B1 = boundary_handler(B1, config)
        v1 = boundary_handler(v1, config)

    if config.numerical_precision == SINGLE_PRECISION:
        tol = 1e-5
    elif config.numerical_precision == DOUBLE_PRECISION:
        tol = 1e-10
    else:
        raise ValueError("Unknown numerical precision.")

    Bk, vk, Bkp1, vkp1, it = B0, v0, B1, v1, 0
    while True:
        change = max(xp.to_float(xp.amax(_norm0(Bk - Bkp1))), xp.to_float(xp.amax(_norm0(vk - vkp1))))
        if not ((change > tol) and (it < MAX_FIXED_POINT_ITERATIONS)):
            break
        Bk, vk = Bkp1, vkp1
        if config.fv_magnetic_integrator == IMPLICIT_MIDPOINT:
            aB, av = (Bk + B) / 2, (vk + velocity) / 2
        elif config.fv_magnetic_integrator == IMPLICIT_EULER:
            aB, av = Bk, vk
        else:
            raise ValueError("unknown magnetic integrator")
        phiA, phiB = phi(av, aB)
        Bkp1 = B - dt * phiA
        vkp1 = velocity - dt * phiB
        if ghost:
            Bkp1 = boundary_handler(Bkp1, config)
            vkp1 = boundary_handler(vkp1, config)
        it += 1
    Bn, vn = Bkp1, vkp1

    vabs = _norm0(velocity)
    vnabs = _norm0(vn)
    E = total_energy_from_primitives(density, vabs, gas[rv.pressure_index], 5 / 3)
    E = E - 0.5 * density * vabs ** 2 + 0.5 * density * vnabs ** 2
    p_new = pressure_from_energy(E, density, vnabs, 5 / 3)
    gas = xp.copy(gas)
    if dims == 2:
        gas[rv.velocity_index.x: rv.velocity_index.x + 2] = vn[:2]
    else:
        gas[rv.velocity_index.x: rv.velocity_index.x + 3] = vn
    gas[rv.pressure_index] = p_new
    if return_iterations:
        return Bn, gas, it
    return Bn, gas


def evolve_state_fv(P, dt, gamma, config, rv, stats=None, C_cfl=None, G=1.0):
    """evolve_state.py:497-600 (unsplit or split gas scheme; MHD via the Pang-Wu split).
    C_cfl is needed by the VAN_ALBADA_PP reconstruction only, G by self-gravity."""
    if not config.mhd:
        return evolve_gas(P, dt, gamma, config, rv, C_cfl, G)
    if config.dimensionality < 2:
        raise ValueError("MHD currently not supported in 1D.")
    rv_gas = rv._replace(num_vars=rv.num_vars - 3)
    gas = P[:-3]
    B = P[-3:]
    gas = evolve_gas(gas, dt / 2, gamma, config, rv_gas, C_cfl, G)
    B, gas, it = magnetic_update(B, gas, config.grid_spacing, dt, config, rv, return_iterations=True)
    if stats is not None:
        stats.append(it)
    gas = evolve_gas(gas, dt / 2, gamma, config, rv_gas, C_cfl, G)
    return xp.concatenate([gas, B], axis=0)


# --------------------------------------------------------------- CFL dt

def cfl_time_step(P, dx, dt_max, gamma, config, rv, C_cfl):
    """_finite_volume/_timestep_estimation/_timestep_estimator.py:95-218."""
    dims = config.dimensionality
    rho = P[rv.density_index]
    p = P[rv.pressure_index]
    if config.split == UNSPLIT:
        c = speed_of_sound(rho, p, gamma)
        total = None
        for axis in range(1, dims + 1):
            a = xp.amax(xp.abs(P[axis]) + c) / dx
            total = a if total is None else total + a
        return C_cfl * 1 / total
    # split: wave speeds |u| + c of the cells on either side of every
    # interface along every axis (get_wave_speeds, :40-88), maximum over axes
    c = speed_of_sound(rho, p, gamma)
    w = xp.abs(P[1:dims + 1]) + c
    nd = P.ndim - 1
    best = None
    for axis in range(1, dims + 1):
        lo = [slice(None)] * nd
        hi = [slice(None)] * nd
        lo[axis - 1] = slice(None, -1)
        hi[axis - 1] = slice(1, None)
        wa = w[axis - 1]
        m = xp.maximum(xp.amax(xp.abs(wa[tuple(lo)])), xp.amax(xp.abs(wa[tuple(hi)])))
        best = m if best is None else xp.maximum(best, m)
    dt = C_cfl * dx / best
    if config.use_max_adaptive_timestep:
        dt = xp.minimum(dt, xp.scalar(dt_max, dt) if hasattr(dt, "dtype") else dt_max)
    return dt
