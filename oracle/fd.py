"""Oracle: CPU restatement of the reference's finite-difference WENO-CT path.

TEST INFRASTRUCTURE ONLY (the checker for the CUDA kernels; the product never
imports it).  Restates, operation for operation, the files under
astronomix/_finite_difference/ of leo1200/astronomix 0.5.1 (3D, periodic
roll, ideal MHD, SSPRK(5,4) + constrained transport).

Conserved state rows: rho, mx, my, mz, E, Bx, By, Bz (registry order of a 3D
MHD state).  Spatial array axes 1, 2, 3 = x, y, z.
"""

from ._xp import xp

# registry of a 3D MHD state (variable_registry/registered_variables.py:156-192)
RHO, MX, MY, MZ, EN, BX, BY, BZ = 0, 1, 2, 3, 4, 5, 6, 7
FACE_X, FACE_Y, FACE_Z = 8, 9, 10


# ------------------------------------------------------------ equations

def cons_from_prim(P, gamma):
    """_finite_difference/_fluid_equations/_equations.py:135-170."""
    rho = P[RHO]
    u2 = P[MX] ** 2 + P[MY] ** 2 + P[MZ] ** 2
    p = P[EN]
    b2 = P[BX] ** 2 + P[BY] ** 2 + P[BZ] ** 2
    E = p / (gamma - 1) + 0.5 * rho * u2 + 0.5 * b2
    U = xp.copy(P)
    U[EN] = E
    U[MX:MZ + 1] = rho * P[MX:MZ + 1]
    return U


def prim_from_cons(U, rhomin, pgmin, gamma, enforce_positivity=True):
    """_finite_difference/_fluid_equations/_equations.py:174-222."""
    rho = U[RHO]
    E = U[EN]
    ux = U[MX] / rho
    uy = U[MY] / rho
    uz = U[MZ] / rho
    u2 = ux ** 2 + uy ** 2 + uz ** 2
    b2 = U[BX] ** 2 + U[BY] ** 2 + U[BZ] ** 2
    p = (gamma - 1) * (E - 0.5 * rho * u2 - 0.5 * b2)
    P = xp.copy(U)
    P[EN] = p
    P[MX] = ux
    P[MY] = uy
    P[MZ] = uz
    if enforce_positivity:
        P[RHO] = xp.maximum(P[RHO], rhomin)
        P[EN] = xp.maximum(P[EN], pgmin)
    return P


def enforce_positivity(U, gamma, rhomin, pgmin):
    """_finite_difference/_fluid_equations/_enforce_positivity.py:24-59."""
    rho = xp.maximum(U[RHO], rhomin)
    vx = U[MX] / rho
    vy = U[MY] / rho
    vz = U[MZ] / rho
    b2 = U[BX] ** 2 + U[BY] ** 2 + U[BZ] ** 2
    v2 = vx ** 2 + vy ** 2 + vz ** 2
    p = (gamma - 1.0) * (U[EN] - 0.5 * rho * v2 - 0.5 * b2)
    p = xp.maximum(p, pgmin)
    E = p / (gamma - 1.0) + 0.5 * rho * v2 + 0.5 * b2
    U = xp.copy(U)
    U[RHO] = rho
    U[EN] = E
    return U


def mhd_flux_x(U, rhomin, pgmin, gamma, enforce_pos=True):
    """_finite_difference/_fluid_equations/_fluxes.py:23-69."""
    P = prim_from_cons(U, rhomin, pgmin, gamma, enforce_pos)
    rho, vx, vy, vz = P[RHO], P[MX], P[MY], P[MZ]
    Bx, By, Bz, p = P[BX], P[BY], P[BZ], P[EN]
    b2 = Bx ** 2 + By ** 2 + Bz ** 2
    v2 = vx ** 2 + vy ** 2 + vz ** 2
    ptot = p + 0.5 * b2
    vdotB = vx * Bx + vy * By + vz * Bz
    E = p / (gamma - 1) + 0.5 * rho * v2 + 0.5 * b2
    F = xp.zeros_like(P)
    F[RHO] = rho * vx
    F[MX] = rho * vx ** 2 + ptot - Bx ** 2
    F[MY] = rho * vx * vy - Bx * By
    F[MZ] = rho * vx * vz - Bx * Bz
    F[EN] = (E + ptot) * vx - vdotB * Bx
    F[BX] = F[BX] * 0.0
    F[BY] = By * vx - Bx * vy
    F[BZ] = Bz * vx - Bx * vz
    return F


# ------------------------------------------------------------ eigen system

def _dss(x):
    # _eigen.py:21-24
    return xp.sqrt(xp.maximum(x, 1e-12))


def eigenvalue_blocks(U, gamma, rhomin, pgmin):
    """_finite_difference/_fluid_equations/_eigen.py:28-114 (cell centred)."""
    rho = U[RHO]
    vx = U[MX] / rho
    vy = U[MY] / rho
    vz = U[MZ] / rho
    v2 = vx * vx + vy * vy + vz * vz
    Bx, By, Bz = U[BX], U[BY], U[BZ]
    b2 = Bx * Bx + By * By + Bz * Bz
    pg = (gamma - 1.0) * (U[EN] - 0.5 * (rho * v2 + b2))
    rho = xp.where((rho < rhomin) | (pg < pgmin), xp.maximum(rho, rhomin), rho)
    pg = xp.where((rho < rhomin) | (pg < pgmin), xp.maximum(pg, pgmin), pg)
    cs2 = xp.maximum(0.0, gamma * xp.abs(pg / rho))
    disc = _dss(xp.maximum(0.0, (b2 / rho + cs2) ** 2 - 4.0 * (Bx * Bx) / rho * cs2))
    cf = _dss(xp.maximum(0.0, 0.5 * (b2 / rho + cs2 + disc)))
    ca = _dss(xp.maximum(0.0, (Bx * Bx) / rho))
    cslow = _dss(xp.maximum(0.0, 0.5 * (b2 / rho + cs2 - disc)))
    return vx, cf, ca, cslow


def all_lambdas(U, gamma, rhomin, pgmin):
    """_eigen.py:915-946."""
    vx, cf, ca, cs = eigenvalue_blocks(U, gamma, rhomin, pgmin)
    return xp.stack([vx - cf, vx - ca, vx - cs, vx, vx + cs, vx + ca, vx + cf], axis=0)


def eigenvector_blocks(U, gamma, rhomin, pgmin):
    """_eigen.py:117-337 (interface i+1/2 stored at index i, axis x)."""
    rho = U[RHO]
    vx = U[MX] / rho
    vy = U[MY] / rho
    vz = U[MZ] / rho
    vsq = vx * vx + vy * vy + vz * vz
    Bx, By, Bz = U[BX], U[BY], U[BZ]
    bsq = Bx * Bx + By * By + Bz * Bz
    energy = U[EN]
    pg = (gamma - 1.0) * (energy - 0.5 * (rho * vsq + bsq))
    rho = xp.where((rho < rhomin) | (pg < pgmin), xp.maximum(rho, rhomin), rho)
    pg = xp.where((rho < rhomin) | (pg < pgmin), xp.maximum(pg, pgmin), pg)
    energy = xp.where((rho < rhomin) | (pg < pgmin),
                      pg / (gamma - 1.0) + 0.5 * (rho * vsq + bsq), energy)
    h = (energy + pg) / rho

    def avg(a):
        return 0.5 * (a + xp.roll(a, -1, 0))

    r_i = avg(rho)
    vx_i, vy_i, vz_i = avg(vx), avg(vy), avg(vz)
    bx_i, by_i, bz_i = avg(Bx), avg(By), avg(Bz)
    h_i = avg(h)
    vsq_i = vx_i * vx_i + vy_i * vy_i + vz_i * vz_i
    bsq_i = bx_i * bx_i + by_i * by_i + bz_i * bz_i
    b2r = bsq_i / r_i
    bx2r = (bx_i * bx_i) / r_i
    a2 = (gamma - 1.0) * (h_i - 0.5 * (vsq_i + b2r))
    a = _dss(xp.maximum(0.0, a2))
    disc = (b2r + a2) ** 2 - 4.0 * bx2r * a2
    disc_r = _dss(xp.maximum(0.0, disc))
    cf = _dss(xp.maximum(0.0, 0.5 * (b2r + a2 + disc_r)))
    ca = _dss(xp.maximum(0.0, bx2r))
    cs = _dss(xp.maximum(0.0, 0.5 * (b2r + a2 - disc_r)))
    bt2 = by_i * by_i + bz_i * bz_i
    sgn_bx = xp.where(bx_i >= 0.0, 1.0, -1.0)
    bt2 = xp.maximum(bt2, 1.0e-12)
    bty = xp.where(bt2 >= 1.0e-12, by_i / _dss(bt2), 1.0 / _dss(xp.scalar(2.0, bt2)))
    btz = xp.where(bt2 >= 1.0e-12, bz_i / _dss(bt2), 1.0 / _dss(xp.scalar(2.0, bt2)))
    denom = cf * cf - cs * cs
    denom = xp.maximum(denom, 1.0e-12)
    af = xp.where(denom >= 1.0e-12, _dss(xp.maximum(0.0, a2 - cs * cs)) / _dss(denom), 1.0)
    aslow = xp.where(denom >= 1e-12, _dss(xp.maximum(0.0, cf * cf - a2)) / _dss(denom), 1.0)
    sqrt_rho = _dss(r_i)
    gam0 = 1.0 - gamma
    gam1 = 0.5 * (gamma - 1.0)
    gam2 = (gamma - 2.0) / (gamma - 1.0)
    a2inv = xp.where(a2 > 0.0, 1.0 / a2, 0.0)
    sgn_bt = xp.where(by_i != 0.0, xp.where(by_i >= 0.0, 1.0, -1.0), xp.where(bz_i >= 0.0, 1.0, -1.0))
    a_ge_ca = a >= ca
    return dict(r=r_i, sqrt_rho=sqrt_rho, vx=vx_i, vy=vy_i, vz=vz_i, vsq=vsq_i,
                bx=bx_i, by=by_i, bz=bz_i, bty=bty, btz=btz, sgn_bx=sgn_bx, sgn_bt=sgn_bt,
                a=a, a2=a2, a2inv=a2inv, a_ge_ca=a_ge_ca, cf=cf, ca=ca, cs=cs,
                af=af, aslow=aslow, gam0=gam0, gam1=gam1, gam2=gam2)


def R_col(U, gamma, rhomin, pgmin, col, e=None):
    """_eigen.py:341-622."""
    e = e or eigenvector_blocks(U, gamma, rhomin, pgmin)
    vx, vy, vz, vsq = e["vx"], e["vy"], e["vz"], e["vsq"]
    bty, btz, sbx, sbt = e["bty"], e["btz"], e["sgn_bx"], e["sgn_bt"]
    a, a2, cf, cs, af, aS = e["a"], e["a2"], e["cf"], e["cs"], e["af"], e["aslow"]
    sr, gam2, ge = e["sqrt_rho"], e["gam2"], e["a_ge_ca"]
    R = xp.zeros_like(U[:8])
    if col == 0:
        R[RHO] = af
        R[MX] = af * (vx - cf)
        R[MY] = af * vy + aS * cs * bty * sbx
        R[MZ] = af * vz + aS * cs * btz * sbx
        R[BY] = a * aS * bty / sr
        R[BZ] = a * aS * btz / sr
        R[EN] = af * (cf ** 2 - cf * vx + 0.5 * vsq - gam2 * a2) + aS * cs * (bty * vy + btz * vz) * sbx
        R = xp.where(~ge, R * sbt, R)
    elif col == 1:
        R[RHO] = R[RHO] * 0.0
        R[MY] = -btz
        R[MZ] = bty
        R[BY] = -btz * sbx / sr
        R[BZ] = bty * sbx / sr
        R[EN] = bty * vz - btz * vy
    elif col == 2:
        R[RHO] = aS
        R[MX] = aS * (vx - cs)
        R[MY] = aS * vy - af * cf * bty * sbx
        R[MZ] = aS * vz - af * cf * btz * sbx
        R[BY] = -a * af * bty / sr
        R[BZ] = -a * af * btz / sr
        R[EN] = aS * (cs ** 2 - cs * vx + 0.5 * vsq - gam2 * a2) - af * cf * (bty * vy + btz * vz) * sbx
        R = xp.where(ge, R * sbt, R)
    elif col == 3:
        R[RHO] = R[RHO] * 0.0 + 1.0
        R[MX] = vx
        R[MY] = vy
        R[MZ] = vz
        R[EN] = 0.5 * vsq
    elif col == 4:
        R[RHO] = aS
        R[MX] = aS * (vx + cs)
        R[MY] = aS * vy + af * cf * bty * sbx
        R[MZ] = aS * vz + af * cf * btz * sbx
        R[BY] = -a * af * bty / sr
        R[BZ] = -a * af * btz / sr
        R[EN] = aS * (cs ** 2 + cs * vx + 0.5 * vsq - gam2 * a2) + af * cf * (bty * vy + btz * vz) * sbx
        R = xp.where(ge, R * sbt, R)
    elif col == 5:
        R[MY] = -btz
        R[MZ] = bty
        R[BY] = btz * sbx / sr
        R[BZ] = -bty * sbx / sr
        R[EN] = bty * vz - btz * vy
    elif col == 6:
        R[RHO] = af
        R[MX] = af * (vx + cf)
        R[MY] = af * vy - aS * cs * bty * sbx
        R[MZ] = af * vz - aS * cs * btz * sbx
        R[BY] = a * aS * bty / sr
        R[BZ] = a * aS * btz / sr
        R[EN] = af * (cf ** 2 + cf * vx + 0.5 * vsq - gam2 * a2) - aS * cs * (bty * vy + btz * vz) * sbx
        R = xp.where(~ge, R * sbt, R)
    return R


def L_row(U, gamma, rhomin, pgmin, row, e=None):
    """_eigen.py:626-911."""
    e = e or eigenvector_blocks(U, gamma, rhomin, pgmin)
    vx, vy, vz, vsq = e["vx"], e["vy"], e["vz"], e["vsq"]
    by, bz = e["by"], e["bz"]
    bty, btz, sbx, sbt = e["bty"], e["btz"], e["sgn_bx"], e["sgn_bt"]
    a, a2, a2inv, cf, cs, af, aS = e["a"], e["a2"], e["a2inv"], e["cf"], e["cs"], e["af"], e["aslow"]
    sr, gam0, gam1, ge = e["sqrt_rho"], e["gam0"], e["gam1"], e["a_ge_ca"]
    L = xp.zeros_like(U[:8])
    if row == 0:
        L[RHO] = af * (gam1 * vsq + cf * vx) - aS * cs * (bty * vy + btz * vz) * sbx
        L[MX] = af * (gam0 * vx - cf)
        L[MY] = gam0 * af * vy + aS * cs * bty * sbx
        L[MZ] = gam0 * af * vz + aS * cs * btz * sbx
        L[BY] = gam0 * af * by + a * aS * bty * sr
        L[BZ] = gam0 * af * bz + a * aS * btz * sr
        L[EN] = L[EN] * 0.0 + (-gam0 * af)
        L = 0.5 * L * a2inv
        L = xp.where(~ge, L * sbt, L)
    elif row == 1:
        L[RHO] = btz * vy - bty * vz
        L[MY] = -btz
        L[MZ] = bty
        L[BY] = -btz * sbx * sr
        L[BZ] = bty * sbx * sr
        L = 0.5 * L
    elif row == 2:
        L[RHO] = aS * (gam1 * vsq + cs * vx) + af * cf * (bty * vy + btz * vz) * sbx
        L[MX] = gam0 * aS * vx - aS * cs
        L[MY] = gam0 * aS * vy - af * cf * bty * sbx
        L[MZ] = gam0 * aS * vz - af * cf * btz * sbx
        L[BY] = gam0 * aS * by - a * af * bty * sr
        L[BZ] = gam0 * aS * bz - a * af * btz * sr
        L[EN] = L[EN] * 0.0 + (-gam0 * aS)
        L = 0.5 * L * a2inv
        L = xp.where(ge, L * sbt, L)
    elif row == 3:
        L[RHO] = -a2 / gam0 - 0.5 * vsq
        L[MX] = vx
        L[MY] = vy
        L[MZ] = vz
        L[BY] = by
        L[BZ] = bz
        L[EN] = L[EN] * 0.0 - 1.0
        L = -gam0 * L * a2inv
    elif row == 4:
        L[RHO] = aS * (gam1 * vsq - cs * vx) - af * cf * (bty * vy + btz * vz) * sbx
        L[MX] = aS * (gam0 * vx + cs)
        L[MY] = gam0 * aS * vy + af * cf * bty * sbx
        L[MZ] = gam0 * aS * vz + af * cf * btz * sbx
        L[BY] = gam0 * aS * by - a * af * bty * sr
        L[BZ] = gam0 * aS * bz - a * af * btz * sr
        L[EN] = L[EN] * 0.0 + (-gam0 * aS)
        L = 0.5 * L * a2inv
        L = xp.where(ge, L * sbt, L)
    elif row == 5:
        L[RHO] = btz * vy - bty * vz
        L[MY] = -btz
        L[MZ] = bty
        L[BY] = btz * sbx * sr
        L[BZ] = -bty * sbx * sr
        L = 0.5 * L
    elif row == 6:
        L[RHO] = af * (gam1 * vsq - cf * vx) + aS * cs * (bty * vy + btz * vz) * sbx
        L[MX] = af * (gam0 * vx + cf)
        L[MY] = gam0 * af * vy - aS * cs * bty * sbx
        L[MZ] = gam0 * af * vz - aS * cs * btz * sbx
        L[BY] = gam0 * af * by + a * aS * bty * sr
        L[BZ] = gam0 * af * bz + a * aS * btz * sr
        L[EN] = L[EN] * 0.0 + (-gam0 * af)
        L = 0.5 * L * a2inv
        L = xp.where(~ge, L * sbt, L)
    return L


# -------------------------------------------------------------- WENO

def _dot8(Lr, X):
    # einsum('nxyz,nxyz->xyz'): sum over the 8 rows in row order
    acc = Lr[0] * X[0]
    for n in range(1, 8):
        acc = acc + Lr[n] * X[n]
    return acc


def weno_flux_x(U, rhomin, pgmin, gamma, enforce_pos=True):
    """_finite_difference/_interface_fluxes/_weno.py:112-241.

    Output index i holds the flux at interface i+1/2 along array axis 1.
    """
    eps = 1e-8
    F = mhd_flux_x(U, rhomin, pgmin, gamma, enforce_pos)
    F_int = 1 / 12 * (-xp.roll(F, 1, 1) + 7 * F + 7 * xp.roll(F, -1, 1) - xp.roll(F, -2, 1))
    Fs_ = [xp.roll(F, 2, 1), xp.roll(F, 1, 1), F, xp.roll(F, -1, 1), xp.roll(F, -2, 1), xp.roll(F, -3, 1)]
    Us_ = [xp.roll(U, 2, 1), xp.roll(U, 1, 1), U, xp.roll(U, -1, 1), xp.roll(U, -2, 1), xp.roll(U, -3, 1)]
    vx, cf, ca, cs = eigenvalue_blocks(U, gamma, rhomin, pgmin)
    lambdas = [vx - cf, vx - ca, vx - cs, vx, vx + cs, vx + ca, vx + cf]
    e = eigenvector_blocks(U, gamma, rhomin, pgmin)
    for mode in range(7):
        lam = lambdas[mode]
        Lr = L_row(U, gamma, rhomin, pgmin, mode, e)
        s = [_dot8(Lr, Fm) for Fm in Fs_]
        q = [_dot8(Lr, Um) for Um in Us_]
        d = [s[k + 1] - s[k] for k in range(5)]
        dq = [q[k + 1] - q[k] for k in range(5)]
        lam_st = [xp.roll(lam, 2, 0), xp.roll(lam, 1, 0), lam, xp.roll(lam, -1, 0), xp.roll(lam, -2, 0), xp.roll(lam, -3, 0)]
        amx = xp.abs(lam_st[0])
        for k in range(1, 6):
            amx = xp.maximum(amx, xp.abs(lam_st[k]))

        def phi(a_, b_, c_, d_):
            IS0 = 13.0 * (a_ - b_) ** 2 + 3.0 * (a_ - 3.0 * b_) ** 2
            IS1 = 13.0 * (b_ - c_) ** 2 + 3.0 * (b_ + c_) ** 2
            IS2 = 13.0 * (c_ - d_) ** 2 + 3.0 * (3.0 * c_ - d_) ** 2
            al0 = 1.0 / (eps + IS0) ** 2
            al1 = 6.0 / (eps + IS1) ** 2
            al2 = 3.0 / (eps + IS2) ** 2
            asum = al0 + al1 + al2
            asum = xp.maximum(asum, 1e-14)
            w0 = al0 / asum
            w2 = al2 / asum
            return w0 * (a_ - 2.0 * b_ + c_) / 3.0 + (w2 - 0.5) * (b_ - 2.0 * c_ + d_) / 6.0

        ap, bp, cp, dp = (0.5 * (d[k] + amx * dq[k]) for k in range(4))
        second = phi(ap, bp, cp, dp)
        am = 0.5 * (d[4] - amx * dq[4])
        bm = 0.5 * (d[3] - amx * dq[3])
        cm = 0.5 * (d[2] - amx * dq[2])
        dm = 0.5 * (d[1] - amx * dq[1])
        third = phi(am, bm, cm, dm)
        Fs = -second + third
        Rc = R_col(U, gamma, rhomin, pgmin, mode, e)
        F_int = F_int + Rc * Fs
    return F_int


_SWAP = {1: None, 2: ((MX, MY), (BX, BY), (0, 2, 1, 3)), 3: ((MX, MZ), (BX, BZ), (0, 3, 2, 1))}


def _swap(A, pairs):
    A = xp.copy(A)
    for i, j in pairs:
        ai, aj = xp.copy(A[i]), xp.copy(A[j])
        A[i], A[j] = aj, ai
    return A


def weno_flux(U, axis, rhomin, pgmin, gamma, enforce_pos=True):
    """_weno.py:244-324: y and z fluxes by transpose + component swap."""
    if axis == 1:
        return weno_flux_x(U, rhomin, pgmin, gamma, enforce_pos)
    m, b, perm = _SWAP[axis]
    q = _swap(xp.transpose(U, perm), (m, b))
    Fq = weno_flux_x(q, rhomin, pgmin, gamma, enforce_pos)
    Fq = xp.transpose(Fq, perm)
    return _swap(Fq, (m, b))


# ---------------------------------------------------------- CT and maths

def interp_center_to_face(a, axis):
    # _finite_difference/_maths/_interpolate.py:9-21
    return (-xp.roll(a, 1, axis) + 9 * a + 9 * xp.roll(a, -1, axis) - xp.roll(a, -2, axis)) / 16.0


def interp_face_to_center(f, axis):
    # _interpolate.py:24-36
    return (3 * xp.roll(f, 3, axis) - 25 * xp.roll(f, 2, axis) + 150 * xp.roll(f, 1, axis)
            + 150 * f - 25 * xp.roll(f, -1, axis) + 3 * xp.roll(f, -2, axis)) / 256.0


def point_values_to_averages(q, A, B):
    # _interpolate.py:39-62
    sx = (xp.roll(q, 1, A) - 2 * q + xp.roll(q, -1, A)) / 24.0
    sy = (xp.roll(q, 1, B) - 2 * q + xp.roll(q, -1, B)) / 24.0
    return q + sx + sy


def fd_int6(f, axis):
    # _finite_difference/_maths/_differencing.py:9-30
    c1, c2, c3 = 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0
    return (c1 * (f - xp.roll(f, 1, axis)) + c2 * (xp.roll(f, -1, axis) - xp.roll(f, 2, axis))
            + c3 * (xp.roll(f, -2, axis) - xp.roll(f, 3, axis)))


def interface_field_divergence(bx, by, bz, dx):
    # _differencing.py:33-51
    return fd_int6(bx, 0) / dx + fd_int6(by, 1) / dx + fd_int6(bz, 2) / dx


def initialize_interface_fields(Bx, By, Bz):
    # _finite_difference/_magnetic_update/_constrained_transport.py:202-213
    return interp_center_to_face(Bx, 0), interp_center_to_face(By, 1), interp_center_to_face(Bz, 2)


def ct_rhs(U, Fx, Fy, Fz, dtdx, dtdy, dtdz):
    """_finite_difference/_magnetic_update/_constrained_transport.py:44-155.

    Field axes: 0 = x, 1 = y, 2 = z.
    """
    X, Y, Z = 0, 1, 2
    rho = U[RHO]
    vx, vy, vz = U[MX] / rho, U[MY] / rho, U[MZ] / rho
    Bx, By, Bz = U[BX], U[BY], U[BZ]
    Bx_x = interp_center_to_face(Bx, X)
    By_fx = Fx[BY] + Bx_x * interp_center_to_face(vy, X)
    Bz_fx = Fx[BZ] + Bx_x * interp_center_to_face(vz, X)
    By_y = interp_center_to_face(By, Y)
    Bx_fy = Fy[BX] + By_y * interp_center_to_face(vx, Y)
    Bz_fy = Fy[BZ] + By_y * interp_center_to_face(vz, Y)
    Bz_z = interp_center_to_face(Bz, Z)
    Bx_fz = Fz[BX] + Bz_z * interp_center_to_face(vx, Z)
    By_fz = Fz[BY] + Bz_z * interp_center_to_face(vy, Z)
    Oz = interp_center_to_face(Bx_fy, X) - interp_center_to_face(By_fx, Y)
    Ox = interp_center_to_face(By_fz, Y) - interp_center_to_face(Bz_fy, Z)
    Oy = interp_center_to_face(Bz_fx, Z) - interp_center_to_face(Bx_fz, X)
    Oz = point_values_to_averages(Oz, X, Y)
    Ox = point_values_to_averages(Ox, Y, Z)
    Oy = point_values_to_averages(Oy, X, Z)
    rbx = -dtdy * fd_int6(Oz, Y) + dtdz * fd_int6(Oy, Z)
    rby = -dtdz * fd_int6(Ox, Z) + dtdx * fd_int6(Oz, X)
    rbz = -dtdx * fd_int6(Oy, X) + dtdy * fd_int6(Ox, Y)
    return rbx, rby, rbz


def update_cell_center_fields(U, bx, by, bz):
    """_constrained_transport.py:161-198."""
    b2_old = U[BX] ** 2 + U[BY] ** 2 + U[BZ] ** 2
    U = xp.copy(U)
    U[BX] = interp_face_to_center(bx, 0)
    U[BY] = interp_face_to_center(by, 1)
    U[BZ] = interp_face_to_center(bz, 2)
    b2_new = U[BX] ** 2 + U[BY] ** 2 + U[BZ] ** 2
    U[EN] = U[EN] + 0.5 * (b2_new - b2_old)
    return U


# ------------------------------------------------------------- SSPRK(5,4)

K_RHS = (0.39175222700392, 0.36841059262959, 0.25189177424738, 0.54497475021237, 0.22600748319395)
K_0 = (1.0, 0.44437049406734, 0.62010185138540, 0.17807995410773, -2.081261929715610e-02)
K_CURR = (0.0, 0.55562950593266, 0.37989814861460, 0.82192004589227, 5.03580947213895e-01)
FINAL = (-2.081261929715610e-02, 0.0, 0.51723167208978, -6.518979800418380e-12, 5.03580947213895e-01)


def compute_rhs(q, bx, by, bz, k2, dt, dx, gamma, rhomin, pgmin, enforce_pos=True, wind=None):
    """_finite_difference/_time_integrators/_ssprk.py:197-243.  `wind`:
    (mass-loss rate, final velocity, cell radii, injection cells) for the
    stellar-wind EI source (:230-241), or None."""
    q = update_cell_center_fields(q, bx, by, bz)
    dtdx = k2 * dt / dx
    Fx = weno_flux(q, 1, rhomin, pgmin, gamma, enforce_pos)
    Fy = weno_flux(q, 2, rhomin, pgmin, gamma, enforce_pos)
    Fz = weno_flux(q, 3, rhomin, pgmin, gamma, enforce_pos)
    rbx, rby, rbz = ct_rhs(q, Fx, Fy, Fz, dtdx, dtdx, dtdx)
    rhs_q = -dtdx * ((Fx - xp.roll(Fx, 1, 1)) + (Fy - xp.roll(Fy, 1, 2)) + (Fz - xp.roll(Fz, 1, 3)))
    if wind is not None:
        from .forcing import wind_ei3d_source
        mdot, vinf, r, nic = wind
        rhs_q = rhs_q + wind_ei3d_source(q, k2 * dt, mdot, vinf, r, dx, nic)
    return rhs_q, rbx, rby, rbz


def ssprk4_with_ct(q0, bx0, by0, bz0, gamma, dx, dt, rhomin, pgmin, enforce_pos=True, wind=None):
    """_ssprk.py:178-347."""
    dt_ = xp.scalar(dt, q0)
    k_rhs = [xp.scalar(k, q0) for k in K_RHS]
    k_0 = [xp.scalar(k, q0) for k in K_0]
    k_c = [xp.scalar(k, q0) for k in K_CURR]
    fin = [xp.scalar(k, q0) for k in FINAL]
    q, bx, by, bz = q0, bx0, by0, bz0
    qf, bxf, byf, bzf = fin[0] * q0, fin[0] * bx0, fin[0] * by0, fin[0] * bz0
    for s in range(4):
        if enforce_pos:
            q = enforce_positivity(q, gamma, rhomin, pgmin)
        rq, rbx, rby, rbz = compute_rhs(q, bx, by, bz, k_rhs[s], dt_, dx, gamma, rhomin, pgmin, enforce_pos, wind)
        q = k_0[s] * q0 + k_c[s] * q + rq
        bx = k_0[s] * bx0 + k_c[s] * bx + rbx
        by = k_0[s] * by0 + k_c[s] * by + rby
        bz = k_0[s] * bz0 + k_c[s] * bz + rbz
        f = fin[s + 1]
        qf = qf + q * f
        bxf = bxf + bx * f
        byf = byf + by * f
        bzf = bzf + bz * f
    rq, rbx, rby, rbz = compute_rhs(q, bx, by, bz, k_rhs[4], dt_, dx, gamma, rhomin, pgmin, enforce_pos, wind)
    qf = qf + rq
    bxf = bxf + rbx
    byf = byf + rby
    bzf = bzf + rbz
    qf = update_cell_center_fields(qf, bxf, byf, bzf)
    if enforce_pos:
        qf = enforce_positivity(qf, gamma, rhomin, pgmin)
    return qf, bxf, byf, bzf


def evolve_state_fd(P, dt, gamma, dx, rhomin, pgmin, enforce_pos=True, wind=None):
    """_finite_difference/_state_evolution/_evolve_state.py:25-73."""
    U = cons_from_prim(P[:-3], gamma)
    bx, by, bz = P[FACE_X], P[FACE_Y], P[FACE_Z]
    U, bx, by, bz = ssprk4_with_ct(U, bx, by, bz, gamma, dx, dt, rhomin, pgmin, enforce_pos, wind)
    Pn = prim_from_cons(U, rhomin, pgmin, gamma, enforce_pos)
    return xp.concatenate([Pn, bx[None], by[None], bz[None]], axis=0)


def cfl_time_step_fd(P, dx, dt_max, gamma, C_cfl, rhomin, pgmin):
    """_finite_difference/_timestep_estimation/_timestep_estimator.py:26-91."""
    U = cons_from_prim(P, gamma)
    lx = xp.amax(xp.abs(all_lambdas(U, gamma, rhomin, pgmin)))
    m, b, perm = _SWAP[2]
    qy = _swap(xp.transpose(U, perm), (m, b))
    ly = xp.amax(xp.abs(all_lambdas(qy, gamma, rhomin, pgmin)))
    m, b, perm = _SWAP[3]
    qz = _swap(xp.transpose(U, perm), (m, b))
    lz = xp.amax(xp.abs(all_lambdas(qz, gamma, rhomin, pgmin)))
    dt = C_cfl * dx / (lx + ly + lz)
    return xp.minimum(dt, dt_max)
