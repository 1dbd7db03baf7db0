// Compiled CPU restatement of the reference's finite-difference WENO-CT MHD
// step (leo1200/astronomix 0.5.1, astronomix/_finite_difference/**), with
// OpenMP over the host's cores.
//
// TEST INFRASTRUCTURE AND CPU BASELINE ONLY: the product (astronomix_gb300)
// never links or calls it.  It restates the same formulas as the NumPy
// oracle (oracle/fd.py), in the same order of operations and without
// floating-point contraction (built with -ffp-contract=off), so that the
// FP64 results agree with the oracle to round-off; it is the timed CPU path
// that bench.py's reference arm and cpu_baseline report beside the GPU.
//
// Files restated (astronomix/_finite_difference/):
//   _fluid_equations/_equations.py:135-222      cons <-> prim (with floors)
//   _fluid_equations/_enforce_positivity.py:24-59
//   _fluid_equations/_fluxes.py:23-69            MHD x-flux
//   _fluid_equations/_eigen.py:28-993            eigenvalues, L rows, R columns
//   _interface_fluxes/_weno.py:112-324           WENO flux, y/z by permutation
//   _magnetic_update/_constrained_transport.py:44-213
//   _maths/_interpolate.py, _maths/_differencing.py
//   _time_integrators/_ssprk.py:178-347          SSPRK(5,4) with CT
//   _timestep_estimation/_timestep_estimator.py:26-91
//   time_stepping/time_integration.py:626-678    adaptive dt, exact end time
//
// State layout: state[11][n][n][n] (C order, z fastest): rho, vx, vy, vz, p,
// Bx, By, Bz (cell centred), bx, by, bz (face fields; index i = face i+1/2).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { RHO = 0, MX = 1, MY = 2, MZ = 3, EN = 4, BX = 5, BY = 6, BZ = 7 };

template <typename T>
inline T jmax(T a, T b) {  // jnp.maximum (NaN wins)
  return (a != a) ? a : ((b != b) ? b : (b > a ? b : a));
}
template <typename T>
inline T jmin(T a, T b) {
  return (a != a) ? a : ((b != b) ? b : (b < a ? b : a));
}
template <typename T>
inline T dss(T x) {  // diff_safe_sqrt (_eigen.py:21-24)
  return std::sqrt(jmax(x, T(1e-12)));
}
template <typename T>
inline T sq(T x) {
  return x * x;
}

// row swap that makes axis `ax` (1 = x, 2 = y, 3 = z) the "x" of _weno_flux_x
inline int perm(int ax, int r) {
  if (ax == 2) {
    if (r == MX) return MY;
    if (r == MY) return MX;
    if (r == BX) return BY;
    if (r == BY) return BX;
  } else if (ax == 3) {
    if (r == MX) return MZ;
    if (r == MZ) return MX;
    if (r == BX) return BZ;
    if (r == BZ) return BX;
  }
  return r;
}

template <typename T>
struct Grid {
  int n;
  long long nc;
  long long stride[4];  // element stride of axis 1..3
  std::vector<int> wrap;  // wrap[i + 8] = i mod n for i in [-8, n + 8)
  void init(int n_) {
    n = n_;
    nc = (long long)n * n * n;
    stride[1] = (long long)n * n;
    stride[2] = n;
    stride[3] = 1;
    wrap.resize(n + 16);
    for (int i = -8; i < n + 8; ++i) wrap[i + 8] = ((i % n) + n) % n;
  }
  // cell c = (i, j, k) shifted by `off` (|off| <= 8) along axis ax (1..3), periodic
  long long shift(long long c, int ax, int off) const {
    const long long s = stride[ax];
    const int x = (int)((c / s) % n);
    return c + (long long)(wrap[x + off + 8] - x) * s;
  }
};

// ------------------------------------------------------------ equations

template <typename T>
void prim_to_cons(const T* P, T* U, T g) {  // _equations.py:135-170
  const T rho = P[RHO];
  const T u2 = P[MX] * P[MX] + P[MY] * P[MY] + P[MZ] * P[MZ];
  const T b2 = P[BX] * P[BX] + P[BY] * P[BY] + P[BZ] * P[BZ];
  for (int r = 0; r < 8; ++r) U[r] = P[r];
  U[EN] = P[EN] / (g - T(1)) + T(0.5) * rho * u2 + T(0.5) * b2;
  U[MX] = rho * P[MX];
  U[MY] = rho * P[MY];
  U[MZ] = rho * P[MZ];
}

template <typename T>
void cons_to_prim(const T* U, T* P, T g, T rhomin, T pgmin, bool floors) {  // _equations.py:174-222
  const T rho = U[RHO];
  const T ux = U[MX] / rho, uy = U[MY] / rho, uz = U[MZ] / rho;
  const T u2 = ux * ux + uy * uy + uz * uz;
  const T b2 = U[BX] * U[BX] + U[BY] * U[BY] + U[BZ] * U[BZ];
  const T p = (g - T(1)) * (U[EN] - T(0.5) * rho * u2 - T(0.5) * b2);
  for (int r = 0; r < 8; ++r) P[r] = U[r];
  P[EN] = p;
  P[MX] = ux;
  P[MY] = uy;
  P[MZ] = uz;
  if (floors) {
    P[RHO] = jmax(P[RHO], rhomin);
    P[EN] = jmax(P[EN], pgmin);
  }
}

template <typename T>
void positivity(T* U, T g, T rhomin, T pgmin) {  // _enforce_positivity.py:24-59
  const T rho = jmax(U[RHO], rhomin);
  const T vx = U[MX] / rho, vy = U[MY] / rho, vz = U[MZ] / rho;
  const T b2 = U[BX] * U[BX] + U[BY] * U[BY] + U[BZ] * U[BZ];
  const T v2 = vx * vx + vy * vy + vz * vz;
  T p = (g - T(1)) * (U[EN] - T(0.5) * rho * v2 - T(0.5) * b2);
  p = jmax(p, pgmin);
  U[EN] = p / (g - T(1)) + T(0.5) * rho * v2 + T(0.5) * b2;
  U[RHO] = rho;
}

template <typename T>
void mhd_flux_x(const T* U, T* F, T g, T rhomin, T pgmin, bool floors) {  // _fluxes.py:23-69
  T P[8];
  cons_to_prim(U, P, g, rhomin, pgmin, floors);
  const T rho = P[RHO], vx = P[MX], vy = P[MY], vz = P[MZ];
  const T Bx = P[BX], By = P[BY], Bz = P[BZ], p = P[EN];
  const T b2 = Bx * Bx + By * By + Bz * Bz;
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T ptot = p + T(0.5) * b2;
  const T vdotB = vx * Bx + vy * By + vz * Bz;
  const T E = p / (g - T(1)) + T(0.5) * rho * v2 + T(0.5) * b2;
  F[RHO] = rho * vx;
  F[MX] = rho * (vx * vx) + ptot - Bx * Bx;
  F[MY] = rho * vx * vy - Bx * By;
  F[MZ] = rho * vx * vz - Bx * Bz;
  F[EN] = (E + ptot) * vx - vdotB * Bx;
  F[BX] = T(0);
  F[BY] = By * vx - Bx * vy;
  F[BZ] = Bz * vx - Bx * vz;
}

// floored rho and pressure of the eigen building blocks; every jnp.where
// re-tests its condition on the values already replaced (_eigen.py:61-74)
template <typename T>
void eigen_floors(const T* U, T g, T rhomin, T pgmin, T* rho_, T* v, T* pg_, T* energy_, T* vsq_, T* bsq_) {
  T rho = U[RHO];
  v[0] = U[MX] / rho;
  v[1] = U[MY] / rho;
  v[2] = U[MZ] / rho;
  const T vsq = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  const T bsq = U[BX] * U[BX] + U[BY] * U[BY] + U[BZ] * U[BZ];
  T energy = U[EN];
  T pg = (g - T(1)) * (energy - T(0.5) * (rho * vsq + bsq));
  rho = ((rho < rhomin) || (pg < pgmin)) ? jmax(rho, rhomin) : rho;
  pg = ((rho < rhomin) || (pg < pgmin)) ? jmax(pg, pgmin) : pg;
  energy = ((rho < rhomin) || (pg < pgmin)) ? pg / (g - T(1)) + T(0.5) * (rho * vsq + bsq) : energy;
  *rho_ = rho;
  *pg_ = pg;
  *energy_ = energy;
  *vsq_ = vsq;
  *bsq_ = bsq;
}

// _eigen_all_lambdas (_eigen.py:28-114, :915-946) of one cell
template <typename T>
void lambdas(const T* U, T g, T rhomin, T pgmin, T* lam) {
  T rho, v[3], pg, energy, vsq, bsq;
  eigen_floors(U, g, rhomin, pgmin, &rho, v, &pg, &energy, &vsq, &bsq);
  const T Bx = U[BX];
  const T cs2 = jmax(T(0), g * std::fabs(pg / rho));
  const T disc = dss(jmax(T(0), sq(bsq / rho + cs2) - T(4) * (Bx * Bx) / rho * cs2));
  const T cf = dss(jmax(T(0), T(0.5) * (bsq / rho + cs2 + disc)));
  const T ca = dss(jmax(T(0), (Bx * Bx) / rho));
  const T cs = dss(jmax(T(0), T(0.5) * (bsq / rho + cs2 - disc)));
  const T vx = v[0];
  lam[0] = vx - cf;
  lam[1] = vx - ca;
  lam[2] = vx - cs;
  lam[3] = vx;
  lam[4] = vx + cs;
  lam[5] = vx + ca;
  lam[6] = vx + cf;
}

// interface eigenvector blocks (_eigen.py:117-337) from cells i and i+1
template <typename T>
struct Eig {
  T vx, vy, vz, vsq, by, bz, bty, btz, sbx, sbt, a, a2, a2inv, cf, cs, af, as, sr, gam0, gam1, gam2;
  bool ge;
};

template <typename T>
Eig<T> eig_interface(const T* UL, const T* UR, T g, T rhomin, T pgmin) {
  T rl, vl[3], pl, el, vsql, bsql, rr, vr[3], pr, er, vsqr, bsqr;
  eigen_floors(UL, g, rhomin, pgmin, &rl, vl, &pl, &el, &vsql, &bsql);
  eigen_floors(UR, g, rhomin, pgmin, &rr, vr, &pr, &er, &vsqr, &bsqr);
  const T hl = (el + pl) / rl, hr = (er + pr) / rr;
  auto avg = [](T a, T b) { return T(0.5) * (a + b); };
  const T r = avg(rl, rr), vx = avg(vl[0], vr[0]), vy = avg(vl[1], vr[1]), vz = avg(vl[2], vr[2]);
  const T bx = avg(UL[BX], UR[BX]), by = avg(UL[BY], UR[BY]), bz = avg(UL[BZ], UR[BZ]), h = avg(hl, hr);
  const T vsq = vx * vx + vy * vy + vz * vz;
  const T bsq = bx * bx + by * by + bz * bz;
  const T b2r = bsq / r, bx2r = (bx * bx) / r;
  const T a2 = (g - T(1)) * (h - T(0.5) * (vsq + b2r));
  const T a = dss(jmax(T(0), a2));
  const T disc = sq(b2r + a2) - T(4) * bx2r * a2;
  const T disc_r = dss(jmax(T(0), disc));
  const T cf = dss(jmax(T(0), T(0.5) * (b2r + a2 + disc_r)));
  const T ca = dss(jmax(T(0), bx2r));
  const T cs = dss(jmax(T(0), T(0.5) * (b2r + a2 - disc_r)));
  T bt2 = by * by + bz * bz;
  Eig<T> e;
  e.sbx = (bx >= T(0)) ? T(1) : T(-1);
  bt2 = jmax(bt2, T(1e-12));
  e.bty = (bt2 >= T(1e-12)) ? by / dss(bt2) : T(1) / dss(T(2));
  e.btz = (bt2 >= T(1e-12)) ? bz / dss(bt2) : T(1) / dss(T(2));
  T denom = cf * cf - cs * cs;
  denom = jmax(denom, T(1e-12));
  e.af = (denom >= T(1e-12)) ? dss(jmax(T(0), a2 - cs * cs)) / dss(denom) : T(1);
  e.as = (denom >= T(1e-12)) ? dss(jmax(T(0), cf * cf - a2)) / dss(denom) : T(1);
  e.sr = dss(r);
  e.gam0 = T(1) - g;
  e.gam1 = T(0.5) * (g - T(1));
  e.gam2 = (g - T(2)) / (g - T(1));
  e.a2inv = (a2 > T(0)) ? T(1) / a2 : T(0);
  e.sbt = (by != T(0)) ? ((by >= T(0)) ? T(1) : T(-1)) : ((bz >= T(0)) ? T(1) : T(-1));
  e.ge = a >= ca;
  e.vx = vx;
  e.vy = vy;
  e.vz = vz;
  e.vsq = vsq;
  e.by = by;
  e.bz = bz;
  e.a = a;
  e.a2 = a2;
  e.cf = cf;
  e.cs = cs;
  return e;
}

template <typename T>
void L_row(const Eig<T>& e, int row, T* L) {  // _eigen.py:626-911
  const T vx = e.vx, vy = e.vy, vz = e.vz, vsq = e.vsq, bty = e.bty, btz = e.btz, sbx = e.sbx, sbt = e.sbt;
  const T a = e.a, a2 = e.a2, a2inv = e.a2inv, cf = e.cf, cs = e.cs, af = e.af, aS = e.as, sr = e.sr;
  const T gam0 = e.gam0, gam1 = e.gam1;
  for (int r = 0; r < 8; ++r) L[r] = T(0);
  switch (row) {
    case 0:
    case 6: {
      const T s = (row == 0) ? T(1) : T(-1);
      L[RHO] = af * (gam1 * vsq + s * cf * vx) - s * aS * cs * (bty * vy + btz * vz) * sbx;
      L[MX] = af * (gam0 * vx - s * cf);
      L[MY] = gam0 * af * vy + s * aS * cs * bty * sbx;
      L[MZ] = gam0 * af * vz + s * aS * cs * btz * sbx;
      L[BY] = gam0 * af * e.by + a * aS * bty * sr;
      L[BZ] = gam0 * af * e.bz + a * aS * btz * sr;
      L[EN] = -gam0 * af;
      for (int r = 0; r < 8; ++r) L[r] = T(0.5) * L[r] * a2inv;
      if (!e.ge)
        for (int r = 0; r < 8; ++r) L[r] = L[r] * sbt;
      break;
    }
    case 1:
    case 5: {
      const T s = (row == 1) ? T(1) : T(-1);
      L[RHO] = btz * vy - bty * vz;
      L[MY] = -btz;
      L[MZ] = bty;
      L[BY] = -s * btz * sbx * sr;
      L[BZ] = s * bty * sbx * sr;
      for (int r = 0; r < 8; ++r) L[r] = T(0.5) * L[r];
      break;
    }
    case 2:
    case 4: {
      if (row == 2) {
        L[RHO] = aS * (gam1 * vsq + cs * vx) + af * cf * (bty * vy + btz * vz) * sbx;
        L[MX] = gam0 * aS * vx - aS * cs;
        L[MY] = gam0 * aS * vy - af * cf * bty * sbx;
        L[MZ] = gam0 * aS * vz - af * cf * btz * sbx;
      } else {
        L[RHO] = aS * (gam1 * vsq - cs * vx) - af * cf * (bty * vy + btz * vz) * sbx;
        L[MX] = aS * (gam0 * vx + cs);
        L[MY] = gam0 * aS * vy + af * cf * bty * sbx;
        L[MZ] = gam0 * aS * vz + af * cf * btz * sbx;
      }
      L[BY] = gam0 * aS * e.by - a * af * bty * sr;
      L[BZ] = gam0 * aS * e.bz - a * af * btz * sr;
      L[EN] = -gam0 * aS;
      for (int r = 0; r < 8; ++r) L[r] = T(0.5) * L[r] * a2inv;
      if (e.ge)
        for (int r = 0; r < 8; ++r) L[r] = L[r] * sbt;
      break;
    }
    default: {  // 3
      L[RHO] = -a2 / gam0 - T(0.5) * vsq;
      L[MX] = vx;
      L[MY] = vy;
      L[MZ] = vz;
      L[BY] = e.by;
      L[BZ] = e.bz;
      L[EN] = T(-1);
      for (int r = 0; r < 8; ++r) L[r] = -gam0 * L[r] * a2inv;
      break;
    }
  }
}

template <typename T>
void R_col(const Eig<T>& e, int col, T* R) {  // _eigen.py:341-622
  const T vx = e.vx, vy = e.vy, vz = e.vz, vsq = e.vsq, bty = e.bty, btz = e.btz, sbx = e.sbx, sbt = e.sbt;
  const T a = e.a, a2 = e.a2, cf = e.cf, cs = e.cs, af = e.af, aS = e.as, sr = e.sr, gam2 = e.gam2;
  for (int r = 0; r < 8; ++r) R[r] = T(0);
  bool flip = false;
  switch (col) {
    case 0:
    case 6: {
      const T s = (col == 0) ? T(-1) : T(1);
      R[RHO] = af;
      R[MX] = af * (vx + s * cf);
      R[MY] = af * vy - s * aS * cs * bty * sbx;
      R[MZ] = af * vz - s * aS * cs * btz * sbx;
      R[BY] = a * aS * bty / sr;
      R[BZ] = a * aS * btz / sr;
      R[EN] = af * (cf * cf + s * cf * vx + T(0.5) * vsq - gam2 * a2) - s * aS * cs * (bty * vy + btz * vz) * sbx;
      flip = !e.ge;
      break;
    }
    case 1:
    case 5: {
      const T s = (col == 1) ? T(1) : T(-1);
      R[MY] = -btz;
      R[MZ] = bty;
      R[BY] = -s * btz * sbx / sr;
      R[BZ] = s * bty * sbx / sr;
      R[EN] = bty * vz - btz * vy;
      break;
    }
    case 2:
    case 4: {
      const T s = (col == 2) ? T(-1) : T(1);
      R[RHO] = aS;
      R[MX] = aS * (vx + s * cs);
      R[MY] = aS * vy + s * af * cf * bty * sbx;
      R[MZ] = aS * vz + s * af * cf * btz * sbx;
      R[BY] = -a * af * bty / sr;
      R[BZ] = -a * af * btz / sr;
      R[EN] = aS * (cs * cs + s * cs * vx + T(0.5) * vsq - gam2 * a2) + s * af * cf * (bty * vy + btz * vz) * sbx;
      flip = e.ge;
      break;
    }
    default:  // 3
      R[RHO] = T(1);
      R[MX] = vx;
      R[MY] = vy;
      R[MZ] = vz;
      R[EN] = T(0.5) * vsq;
      break;
  }
  if (flip)
    for (int r = 0; r < 8; ++r) R[r] = R[r] * sbt;
}

template <typename T>
T weno_phi(T a, T b, T c, T d) {  // _weno.py:190-205
  const T eps = T(1e-8);
  const T IS0 = T(13) * sq(a - b) + T(3) * sq(a - T(3) * b);
  const T IS1 = T(13) * sq(b - c) + T(3) * sq(b + c);
  const T IS2 = T(13) * sq(c - d) + T(3) * sq(T(3) * c - d);
  const T al0 = T(1) / sq(eps + IS0);
  const T al1 = T(6) / sq(eps + IS1);
  const T al2 = T(3) / sq(eps + IS2);
  T asum = al0 + al1 + al2;
  asum = jmax(asum, T(1e-14));
  const T w0 = al0 / asum, w2 = al2 / asum;
  return w0 * (a - T(2) * b + c) / T(3) + (w2 - T(0.5)) * (b - T(2) * c + d) / T(6);
}

template <typename T>
T dot8(const T* L, const T* X) {  // einsum over the 8 rows in row order
  T acc = L[0] * X[0];
  for (int r = 1; r < 8; ++r) acc = acc + L[r] * X[r];
  return acc;
}

// ------------------------------------------------------------ the step

template <typename T>
struct Stepper {
  Grid<T> G;
  T g, rhomin, pgmin, dx;
  bool floors;
  // work arrays: [rows][nc]
  std::vector<T> q0, q, qf, qc, b0, b, bf, Fx, Fy, Fz, rb, tmp;
  std::vector<T> cellU, cellF, cellL;  // permuted cell data of one axis: [nc][8], [nc][8], [nc][7]

  explicit Stepper(int n) {
    G.init(n);
    const size_t nc = (size_t)G.nc;
    q0.resize(8 * nc), q.resize(8 * nc), qf.resize(8 * nc), qc.resize(8 * nc);
    b0.resize(3 * nc), b.resize(3 * nc), bf.resize(3 * nc), rb.resize(3 * nc);
    Fx.resize(8 * nc), Fy.resize(8 * nc), Fz.resize(8 * nc), tmp.resize(12 * nc);
    cellU.resize(8 * nc), cellF.resize(8 * nc), cellL.resize(7 * nc);
  }

  // _weno_flux_x/_y/_z (_weno.py:112-324): F[r][c] = flux through face c+1/2 along `ax` (lab rows)
  void weno_flux(const T* U, int ax, T* F) {
    const long long nc = G.nc;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      T u[8], f[8];
      for (int r = 0; r < 8; ++r) u[r] = U[perm(ax, r) * nc + c];
      mhd_flux_x(u, f, g, rhomin, pgmin, floors);
      for (int r = 0; r < 8; ++r) {
        cellU[c * 8 + r] = u[r];
        cellF[c * 8 + r] = f[r];
      }
      lambdas(u, g, rhomin, pgmin, &cellL[c * 7]);
    }
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      long long st[6];
      for (int m = 0; m < 6; ++m) st[m] = G.shift(c, ax, m - 2);  // cells i-2 .. i+3
      const T* Fm[6];
      const T* Um[6];
      for (int m = 0; m < 6; ++m) {
        Fm[m] = &cellF[st[m] * 8];
        Um[m] = &cellU[st[m] * 8];
      }
      T Fi[8];
      for (int r = 0; r < 8; ++r)
        Fi[r] = T(1.0 / 12.0) * (-Fm[1][r] + T(7) * Fm[2][r] + T(7) * Fm[3][r] - Fm[4][r]);
      const Eig<T> e = eig_interface(Um[2], Um[3], g, rhomin, pgmin);
      for (int mode = 0; mode < 7; ++mode) {
        T L[8], R[8], s[6], qq[6], d[5], dq[5];
        L_row(e, mode, L);
        for (int m = 0; m < 6; ++m) {
          s[m] = dot8(L, Fm[m]);
          qq[m] = dot8(L, Um[m]);
        }
        for (int k = 0; k < 5; ++k) {
          d[k] = s[k + 1] - s[k];
          dq[k] = qq[k + 1] - qq[k];
        }
        T amx = std::fabs(cellL[st[0] * 7 + mode]);
        for (int m = 1; m < 6; ++m) amx = jmax(amx, std::fabs(cellL[st[m] * 7 + mode]));
        const T second = weno_phi(T(0.5) * (d[0] + amx * dq[0]), T(0.5) * (d[1] + amx * dq[1]),
                                  T(0.5) * (d[2] + amx * dq[2]), T(0.5) * (d[3] + amx * dq[3]));
        const T third = weno_phi(T(0.5) * (d[4] - amx * dq[4]), T(0.5) * (d[3] - amx * dq[3]),
                                 T(0.5) * (d[2] - amx * dq[2]), T(0.5) * (d[1] - amx * dq[1]));
        const T Fs = -second + third;
        R_col(e, mode, R);
        for (int r = 0; r < 8; ++r) Fi[r] = Fi[r] + R[r] * Fs;
      }
      for (int r = 0; r < 8; ++r) F[perm(ax, r) * nc + c] = Fi[r];
    }
  }

  // interp_center_to_face (_interpolate.py:9-21) along ax
  T c2f(const T* a, long long c, int ax) const {
    return (-a[G.shift(c, ax, -1)] + T(9) * a[c] + T(9) * a[G.shift(c, ax, 1)] - a[G.shift(c, ax, 2)]) / T(16);
  }
  // interp_face_to_center (_interpolate.py:24-36)
  T f2c(const T* f, long long c, int ax) const {
    return (T(3) * f[G.shift(c, ax, -3)] - T(25) * f[G.shift(c, ax, -2)] + T(150) * f[G.shift(c, ax, -1)] +
            T(150) * f[c] - T(25) * f[G.shift(c, ax, 1)] + T(3) * f[G.shift(c, ax, 2)]) /
           T(256);
  }
  // finite_difference_int6 (_differencing.py:9-30)
  T fd6(const T* f, long long c, int ax) const {
    const T c1 = T(75.0 / 64.0), c2 = T(-25.0 / 384.0), c3 = T(3.0 / 640.0);
    return c1 * (f[c] - f[G.shift(c, ax, -1)]) + c2 * (f[G.shift(c, ax, 1)] - f[G.shift(c, ax, -2)]) +
           c3 * (f[G.shift(c, ax, 2)] - f[G.shift(c, ax, -3)]);
  }

  // update_cell_center_fields (_constrained_transport.py:161-198): out = U with refreshed B and E
  void ucc(const T* U, const T* bx, const T* by, const T* bz, T* out) {
    const long long nc = G.nc;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      const T b2o = U[BX * nc + c] * U[BX * nc + c] + U[BY * nc + c] * U[BY * nc + c] + U[BZ * nc + c] * U[BZ * nc + c];
      for (int r = 0; r < 8; ++r) out[r * nc + c] = U[r * nc + c];
      const T Bx = f2c(bx, c, 1), By = f2c(by, c, 2), Bz = f2c(bz, c, 3);
      out[BX * nc + c] = Bx;
      out[BY * nc + c] = By;
      out[BZ * nc + c] = Bz;
      const T b2n = Bx * Bx + By * By + Bz * Bz;
      out[EN * nc + c] = U[EN * nc + c] + T(0.5) * (b2n - b2o);
    }
  }

  // constrained_transport_rhs (_constrained_transport.py:44-155) into rb[3][nc]
  void ct_rhs(const T* U, T dtdx) {
    const long long nc = G.nc;
    T* vel = tmp.data();          // 3 rows
    T* M = tmp.data() + 3 * nc;   // 6 rows: By_fx Bz_fx Bx_fy Bz_fy Bx_fz By_fz
    T* O = tmp.data() + 9 * nc;   // 3 rows: Ox Oy Oz
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      const T rho = U[RHO * nc + c];
      vel[c] = U[MX * nc + c] / rho;
      vel[nc + c] = U[MY * nc + c] / rho;
      vel[2 * nc + c] = U[MZ * nc + c] / rho;
    }
    const T* Bx = U + BX * nc;
    const T* By = U + BY * nc;
    const T* Bz = U + BZ * nc;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      const T Bx_x = c2f(Bx, c, 1), By_y = c2f(By, c, 2), Bz_z = c2f(Bz, c, 3);
      M[c] = Fx[BY * nc + c] + Bx_x * c2f(vel + nc, c, 1);
      M[nc + c] = Fx[BZ * nc + c] + Bx_x * c2f(vel + 2 * nc, c, 1);
      M[2 * nc + c] = Fy[BX * nc + c] + By_y * c2f(vel, c, 2);
      M[3 * nc + c] = Fy[BZ * nc + c] + By_y * c2f(vel + 2 * nc, c, 2);
      M[4 * nc + c] = Fz[BX * nc + c] + Bz_z * c2f(vel, c, 3);
      M[5 * nc + c] = Fz[BY * nc + c] + Bz_z * c2f(vel + nc, c, 3);
    }
    T* OM = vel;  // point values (velocities no longer needed)
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      OM[2 * nc + c] = c2f(M + 2 * nc, c, 1) - c2f(M, c, 2);          // Oz
      OM[c] = c2f(M + 5 * nc, c, 2) - c2f(M + 3 * nc, c, 3);          // Ox
      OM[nc + c] = c2f(M + nc, c, 3) - c2f(M + 4 * nc, c, 1);         // Oy
    }
    auto avg = [&](const T* q_, long long c, int A, int B) {  // point_values_to_averages (_interpolate.py:39-62)
      const T sx = (q_[G.shift(c, A, -1)] - T(2) * q_[c] + q_[G.shift(c, A, 1)]) / T(24);
      const T sy = (q_[G.shift(c, B, -1)] - T(2) * q_[c] + q_[G.shift(c, B, 1)]) / T(24);
      return q_[c] + sx + sy;
    };
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      O[2 * nc + c] = avg(OM + 2 * nc, c, 1, 2);
      O[c] = avg(OM, c, 2, 3);
      O[nc + c] = avg(OM + nc, c, 1, 3);
    }
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      const T* Ox = O;
      const T* Oy = O + nc;
      const T* Oz = O + 2 * nc;
      rb[c] = -dtdx * fd6(Oz, c, 2) + dtdx * fd6(Oy, c, 3);
      rb[nc + c] = -dtdx * fd6(Ox, c, 3) + dtdx * fd6(Oz, c, 1);
      rb[2 * nc + c] = -dtdx * fd6(Oy, c, 1) + dtdx * fd6(Ox, c, 2);
    }
  }

  // compute_rhs (_ssprk.py:197-243): rhs of q into `rq` (8 rows), faces into rb
  void compute_rhs(const T* qq, const T* bb, T k2, T dt, T* rq) {
    const long long nc = G.nc;
    ucc(qq, bb, bb + nc, bb + 2 * nc, qc.data());
    const T dtdx = k2 * dt / dx;
    weno_flux(qc.data(), 1, Fx.data());
    weno_flux(qc.data(), 2, Fy.data());
    weno_flux(qc.data(), 3, Fz.data());
    ct_rhs(qc.data(), dtdx);
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      const long long cx = G.shift(c, 1, -1), cy = G.shift(c, 2, -1), cz = G.shift(c, 3, -1);
      for (int r = 0; r < 8; ++r)
        rq[r * nc + c] = -dtdx * ((Fx[r * nc + c] - Fx[r * nc + cx]) + (Fy[r * nc + c] - Fy[r * nc + cy]) +
                                  (Fz[r * nc + c] - Fz[r * nc + cz]));
    }
  }

  // _evolve_state_fd (_evolve_state.py:25-73) with _ssprk4_with_ct (_ssprk.py:178-347)
  void step(T* P, T dt) {
    static const double K_RHS[5] = {0.39175222700392, 0.36841059262959, 0.25189177424738, 0.54497475021237,
                                    0.22600748319395};
    static const double K_0[5] = {1.0, 0.44437049406734, 0.62010185138540, 0.17807995410773,
                                  -2.081261929715610e-02};
    static const double K_C[5] = {0.0, 0.55562950593266, 0.37989814861460, 0.82192004589227,
                                  5.03580947213895e-01};
    static const double FIN[5] = {-2.081261929715610e-02, 0.0, 0.51723167208978, -6.518979800418380e-12,
                                  5.03580947213895e-01};
    const long long nc = G.nc;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      T p[8], u[8];
      for (int r = 0; r < 8; ++r) p[r] = P[r * nc + c];
      prim_to_cons(p, u, g);
      for (int r = 0; r < 8; ++r) {
        q0[r * nc + c] = u[r];
        q[r * nc + c] = u[r];
        qf[r * nc + c] = T(FIN[0]) * u[r];
      }
      for (int r = 0; r < 3; ++r) {
        b0[r * nc + c] = P[(8 + r) * nc + c];
        b[r * nc + c] = P[(8 + r) * nc + c];
        bf[r * nc + c] = T(FIN[0]) * P[(8 + r) * nc + c];
      }
    }
    std::vector<T> rq(8 * nc);
    for (int s = 0; s < 4; ++s) {
      if (floors) {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < nc; ++c) {
          T u[8];
          for (int r = 0; r < 8; ++r) u[r] = q[r * nc + c];
          positivity(u, g, rhomin, pgmin);
          q[RHO * nc + c] = u[RHO];
          q[EN * nc + c] = u[EN];
        }
      }
      compute_rhs(q.data(), b.data(), T(K_RHS[s]), dt, rq.data());
      const T k0 = T(K_0[s]), kc = T(K_C[s]), f = T(FIN[s + 1]);
#pragma omp parallel for schedule(static)
      for (long long c = 0; c < nc; ++c) {
        for (int r = 0; r < 8; ++r) {
          const long long i = r * nc + c;
          q[i] = k0 * q0[i] + kc * q[i] + rq[i];
          qf[i] = qf[i] + q[i] * f;
        }
        for (int r = 0; r < 3; ++r) {
          const long long i = r * nc + c;
          b[i] = k0 * b0[i] + kc * b[i] + rb[i];
          bf[i] = bf[i] + b[i] * f;
        }
      }
    }
    compute_rhs(q.data(), b.data(), T(K_RHS[4]), dt, rq.data());
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      for (int r = 0; r < 8; ++r) qf[r * nc + c] = qf[r * nc + c] + rq[r * nc + c];
      for (int r = 0; r < 3; ++r) bf[r * nc + c] = bf[r * nc + c] + rb[r * nc + c];
    }
    ucc(qf.data(), bf.data(), bf.data() + nc, bf.data() + 2 * nc, qc.data());
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < nc; ++c) {
      T u[8], p[8];
      for (int r = 0; r < 8; ++r) u[r] = qc[r * nc + c];
      if (floors) positivity(u, g, rhomin, pgmin);
      cons_to_prim(u, p, g, rhomin, pgmin, floors);
      for (int r = 0; r < 8; ++r) P[r * nc + c] = p[r];
      for (int r = 0; r < 3; ++r) P[(8 + r) * nc + c] = bf[r * nc + c];
    }
  }

  // _cfl_time_step_fd (_timestep_estimator.py:26-91)
  double cfl(const T* P, double C_cfl, double dt_max) {
    const long long nc = G.nc;
    double m[3] = {0.0, 0.0, 0.0};
    bool nan = false;
    for (int ax = 1; ax <= 3; ++ax) {
      T best = T(0);
      bool bad = false;
#pragma omp parallel
      {
        T loc = T(0);
        bool lbad = false;
#pragma omp for schedule(static) nowait
        for (long long c = 0; c < nc; ++c) {
          T p[8], u[8], up[8], lam[7];
          for (int r = 0; r < 8; ++r) p[r] = P[r * nc + c];
          prim_to_cons(p, u, g);
          for (int r = 0; r < 8; ++r) up[r] = u[perm(ax, r)];
          lambdas(up, g, rhomin, pgmin, lam);
          for (int k = 0; k < 7; ++k) {
            const T a = std::fabs(lam[k]);
            if (a != a) lbad = true;
            loc = std::max(loc, a);
          }
        }
#pragma omp critical
        {
          best = std::max(best, loc);
          bad = bad || lbad;
        }
      }
      m[ax - 1] = (double)best;
      nan = nan || bad;
    }
    if (nan) return NAN;
    const double dt = C_cfl * (double)dx / (m[0] + m[1] + m[2]);
    return jmin(dt, dt_max);
  }
};

template <typename T>
int run(int n, double dx, double gamma, double rhomin, double pgmin, double C_cfl, double dt_max, double t_end,
        int exact_end_time, int enforce_positivity, int64_t max_steps, T* state, double* t_out, int64_t* steps_out) {
  Stepper<T> S(n);
  S.g = T(gamma);
  S.rhomin = T(rhomin);
  S.pgmin = T(pgmin);
  S.dx = T(dx);
  S.floors = enforce_positivity != 0;
  double t = 0.0;
  int64_t steps = 0;
  while (steps < max_steps && t < t_end) {
    double dt = S.cfl(state, C_cfl, dt_max);
    if (exact_end_time) dt = jmin(dt, t_end - t);
    S.step(state, T(dt));
    t = t + dt;
    ++steps;
  }
  *t_out = t;
  *steps_out = steps;
  return 0;
}

}  // namespace

extern "C" {

// Runs at most max_steps adaptive FD steps of `state` (11 x n^3 values of
// dtype 0 = float32 / 1 = float64) in place, stopping at t_end (dt clipped to
// the end time when exact_end_time).  nthreads > 0 sets the OpenMP threads.
int amxref_fd_run(int dtype, int n, double dx, double gamma, double rhomin, double pgmin, double C_cfl,
                  double dt_max, double t_end, int exact_end_time, int enforce_positivity, int64_t max_steps,
                  void* state, double* t_out, int64_t* steps_out, int nthreads) {
  if (n < 4 || !state || !t_out || !steps_out) return 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  if (dtype == 0)
    return run<float>(n, dx, gamma, rhomin, pgmin, C_cfl, dt_max, t_end, exact_end_time, enforce_positivity,
                      max_steps, static_cast<float*>(state), t_out, steps_out);
  return run<double>(n, dx, gamma, rhomin, pgmin, C_cfl, dt_max, t_end, exact_end_time, enforce_positivity,
                     max_steps, static_cast<double*>(state), t_out, steps_out);
}

// Threads OpenMP will use.
int amxref_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
