// Compiled CPU restatement of the reference's finite-volume MHD step
// (leo1200/astronomix 0.5.1, astronomix/_finite_volume/**), with OpenMP over
// the host's cores.
//
// TEST INFRASTRUCTURE AND CPU BASELINE ONLY: the product (astronomix_gb300)
// never links or calls it.  It restates the NumPy oracle (oracle/fv.py,
// oracle/driver.py with FP64 time) in the same order of operations and
// without floating-point contraction (built with -ffp-contract=off), so that
// its results agree with the oracle to round-off; bench.py times it beside
// the GPU as the compiled CPU baseline of the FV workload.
//
// Scope: 2D and 3D, every boundary periodic, the unsplit SSP-RK2 scheme with
// the limited-linear reconstruction (MINMOD, OSHER, DOUBLE_MINMOD, SUPERBEE,
// VAN_ALBADA), HLL, HLLC or Lax-Friedrichs fluxes, hydro or MHD with the
// Pang-Wu split (implicit midpoint or implicit Euler fixed point).
//
// Files restated (astronomix/_finite_volume/):
//   _fluid_equations/_equations.py:24-280        prim <-> cons, sound speed
//   _fluid_equations/_fluxes.py:25-93              Euler flux
//   _state_evolution/limiters.py, limited_gradients.py:22-88
//   _state_evolution/reconstruction.py:399-431     unsplit interface states
//   _riemann_solver/hll.py:36-261, _lax_friedrichs.py:21-78
//   _state_evolution/evolve_state.py:339-600      unsplit stage, RK2, Pang-Wu
//   _magnetic_update/_magnetic_field_update.py:37-242, _vector_maths.py
//   _timestep_estimation/_timestep_estimator.py:95-128
//   time_stepping/time_integration.py:626-678      adaptive dt, exact end time
//
// State layout: state[nv][n]^dim (C order, last axis fastest): rho, v_x,
// v_y (, v_z), p (, B_x, B_y, B_z).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T>
inline T jmax(T a, T b) {  // jnp.maximum (NaN wins)
  return (a != a) ? a : ((b != b) ? b : (b > a ? b : a));
}
template <typename T>
inline T jmin(T a, T b) {
  return (a != a) ? a : ((b != b) ? b : (b < a ? b : a));
}
template <typename T>
inline T sgn(T x) {  // jnp.sign
  return x > T(0) ? T(1) : (x < T(0) ? T(-1) : (x == x ? T(0) : x));
}

enum { L_MINMOD = 0, L_OSHER = 1, L_DOUBLE_MINMOD = 2, L_SUPERBEE = 3, L_VAN_ALBADA = 4 };
enum { R_HLL = 0, R_HLLC = 1, R_LF = 3 };

struct Geo {
  int dim, n;
  long long nc;
  long long stride[3];  // element stride of axis 0..dim-1
  void init(int d, int n_) {
    dim = d;
    n = n_;
    nc = 1;
    for (int k = 0; k < d; ++k) nc *= n;
    stride[d - 1] = 1;
    for (int k = d - 2; k >= 0; --k) stride[k] = stride[k + 1] * n;
  }
  // the cell `off` (|off| <= n) away from c along axis k, periodic
  long long shift(long long c, int k, int off) const {
    const long long s = stride[k];
    const int x = (int)((c / s) % n);
    int y = x + off;
    if (y < 0) y += n;
    if (y >= n) y -= n;
    return c + (long long)(y - x) * s;
  }
};

// ------------------------------------------------------------ equations

template <typename T>
inline T abs_velocity(const T* q, int dim) {  // get_absolute_velocity
  if (dim == 2) return std::sqrt(q[1] * q[1] + q[2] * q[2]);
  return std::sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + T(1e-20));
}
template <typename T>
inline T total_energy(T rho, T u, T p, T g) {
  return p / (g - T(1)) + T(0.5) * rho * (u * u);
}
template <typename T>
inline T pressure_from_energy(T E, T rho, T u, T g) {
  const T e = E / rho - T(0.5) * (u * u);
  return (g - T(1)) * rho * e;
}
template <typename T>
inline T sound_speed(T rho, T p, T g) {
  return std::sqrt(g * p / rho);
}
template <typename T>
inline void prim_to_cons(const T* q, T* U, T g, int dim) {
  const T rho = q[0];
  const T u = abs_velocity(q, dim);
  U[0] = rho;
  for (int a = 1; a <= dim; ++a) U[a] = rho * q[a];
  U[dim + 1] = total_energy(rho, u, q[dim + 1], g);
}
template <typename T>
inline void cons_to_prim(const T* U, T* q, T g, int dim) {
  const T rho = U[0];
  q[0] = rho;
  T s = T(0);
  for (int a = 1; a <= dim; ++a) {
    q[a] = U[a] / rho;
    s = (a == 1) ? q[a] * q[a] : s + q[a] * q[a];
  }
  const T u = std::sqrt(s + T(1e-20));
  q[dim + 1] = pressure_from_energy(U[dim + 1], rho, u, g);
}
template <typename T>
inline void euler_flux(const T* q, int d, T g, int dim, T* F) {
  const T rho = q[0], p = q[dim + 1], ud = q[d];
  const T E = total_energy(rho, abs_velocity(q, dim), p, g);
  F[0] = ud * rho;
  for (int a = 1; a <= dim; ++a) F[a] = ud * (q[a] * rho);
  F[dim + 1] = ud * (p + E);
  F[d] = F[d] + p;
}

// ------------------------------------------------------------ reconstruction

template <typename T>
inline T minmod(T a, T b) {
  return T(0.5) * (sgn(a) + sgn(b)) * jmin(std::fabs(a), std::fabs(b));
}
// eps3dx: the VAN_ALBADA epsilon 3 dx, formed in FP64 and rounded to T
template <typename T>
inline T limited(T bd, T fd, int lim, T eps3dx) {
  switch (lim) {
    case L_MINMOD:
      return minmod(bd, fd);
    case L_OSHER: {
      const T eps = T(1e-11);
      const T gg = (std::fabs(bd) > eps) ? fd / (bd + eps) : T(0);
      return jmax(T(0), jmin(T(1.3), gg)) * bd;
    }
    case L_DOUBLE_MINMOD: {
      if (!(bd * fd > T(0))) return T(0);
      const T a = (bd + fd) / T(2), b = T(2) * bd, c = T(2) * fd;
      const bool same = (sgn(a) == sgn(b)) && (sgn(b) == sgn(c));
      return same ? sgn(a) * jmin(std::fabs(a), jmin(std::fabs(b), std::fabs(c))) : T(0);
    }
    case L_SUPERBEE: {
      if (!(bd * fd > T(0))) return T(0);
      const T mx = T(0.5) * (sgn(bd) + sgn(fd)) * jmax(std::fabs(bd), std::fabs(fd));
      return minmod(mx, minmod(T(2) * bd, T(2) * fd));
    }
    default: {
      const T eps = eps3dx;
      return ((fd * fd + eps) * bd + (bd * bd + eps) * fd) / (fd * fd + bd * bd + T(2) * eps);
    }
  }
}

// ------------------------------------------------------------ Riemann solvers

template <typename T>
inline void hll(const T* qL, const T* qR, int d, T g, int dim, T* F) {
  const int NV = dim + 2, E = dim + 1;
  const T cL = sound_speed(qL[0], qL[E], g), cR = sound_speed(qR[0], qR[E], g);
  T FL[5], FR[5], UL[5], UR[5];
  euler_flux(qL, d, g, dim, FL);
  euler_flux(qR, d, g, dim, FR);
  const T SR = jmax(jmax(qL[d] + cL, qR[d] + cR), T(0));
  const T SL = jmin(jmin(qL[d] - cL, qR[d] - cR), T(0));
  prim_to_cons(qL, UL, g, dim);
  prim_to_cons(qR, UR, g, dim);
  for (int v = 0; v < NV; ++v) F[v] = (SR * FL[v] - SL * FR[v] + SL * SR * (UR[v] - UL[v])) / (SR - SL);
}

template <typename T>
inline void hllc(const T* qL, const T* qR, int d, T g, int dim, T* F) {
  const int NV = dim + 2, E = dim + 1;
  const T rhoL = qL[0], uL = qL[d], pL = qL[E];
  const T rhoR = qR[0], uR = qR[d], pR = qR[E];
  const T cL = sound_speed(rhoL, pL, g), cR = sound_speed(rhoR, pR, g);
  T FL[5], FR[5], UL[5], UR[5], USL[5], USR[5];
  euler_flux(qL, d, g, dim, FL);
  euler_flux(qR, d, g, dim, FR);
  const T sL = std::sqrt(rhoL), sR = std::sqrt(rhoR);
  const T u_hat = (sL * uL + sR * uR) / (sL + sR);
  const T c_hat_sq = (cL * cL * sL + cR * cR * sR) / (sL + sR) +
                     T(0.5) * (sL * sR / ((sL + sR) * (sL + sR))) * ((uR - uL) * (uR - uL));
  const T c_hat = std::sqrt(c_hat_sq);
  const T SL = jmin(uL - cL, u_hat - c_hat);
  const T SR = jmax(uR + cR, u_hat + c_hat);
  const T S_star = (pR - pL + rhoL * uL * (SL - uL) - rhoR * uR * (SR - uR)) / (rhoL * (SL - uL) - rhoR * (SR - uR));
  prim_to_cons(qL, UL, g, dim);
  prim_to_cons(qR, UR, g, dim);
  for (int v = 0; v < NV; ++v) { USL[v] = UL[v]; USR[v] = UR[v]; }
  USL[d] = rhoL * S_star;
  USL[E] = USL[E] + (S_star - uL) * (rhoL * S_star + pL / (SL - uL));
  USR[d] = rhoR * S_star;
  USR[E] = USR[E] + (S_star - uR) * (rhoR * S_star + pR / (SR - uR));
  const T aS = std::fabs(S_star);
  for (int v = 0; v < NV; ++v) {
    const T usl = USL[v] * (SL - uL) / (SL - S_star), usr = USR[v] * (SR - uR) / (SR - S_star);
    const T Fs = T(0.5) * (FL[v] + FR[v]) + T(0.5) * (SL * (usl - UL[v]) + aS * (usl - usr) + SR * (usr - UR[v]));
    const T f = (SL >= T(0)) ? FL[v] : Fs;
    F[v] = (SR <= T(0)) ? FR[v] : f;
  }
}

template <typename T>
inline void lax_friedrichs(const T* qL, const T* qR, int d, T g, int dim, T alpha, T* F) {
  const int NV = dim + 2;
  T FL[5], FR[5], UL[5], UR[5];
  prim_to_cons(qL, UL, g, dim);
  prim_to_cons(qR, UR, g, dim);
  euler_flux(qL, d, g, dim, FL);
  euler_flux(qR, d, g, dim, FR);
  for (int v = 0; v < NV; ++v) F[v] = T(0.5) * (FL[v] + FR[v]) - T(0.5) * alpha * (UR[v] - UL[v]);
}

// ------------------------------------------------------------ hydro stage

struct Cfg {
  int dim, n, limiter, riemann, mhd, midpoint;
  double dx, gamma, C_cfl, t_end, tol;
  int exact_end_time;
};

// One unsplit stage (evolve_state.py:339-414): U = cons(P); per axis the
// interface states of reconstruction.py:399-431, the Riemann flux and
// U += (1/dx)(F[i] - F[i+1]) dt; returns prim(U) in out.
template <typename T>
void stage(const Cfg& c, const Geo& G, const T* P, T* out, T dt, std::vector<T>& Ubuf, std::vector<T>& Dbuf,
           std::vector<T>& Fbuf) {
  const int dim = c.dim, NV = dim + 2;
  const long long nc = G.nc;
  const T g = T(c.gamma), dxT = T(c.dx), inv_dx = T(1.0 / c.dx), eps3dx = T(3.0 * c.dx);
  T* U = Ubuf.data();
  T* D = Dbuf.data();  // [NV][nc] g * dx / 2 of the current axis
  T* F = Fbuf.data();  // [NV][nc] flux at face i (between cells i-1 and i)
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < nc; ++i) {
    T q[5], u[5];
    for (int v = 0; v < NV; ++v) q[v] = P[v * nc + i];
    prim_to_cons(q, u, g, dim);
    for (int v = 0; v < NV; ++v) U[v * nc + i] = u[v];
  }
  for (int ax = 0; ax < dim; ++ax) {
    const int d = ax + 1;
    T alpha = T(0);
    if (c.riemann == R_LF) {  // the stage state's global max |u_d| + c
      T m = T(0);
      bool first = true;
#pragma omp parallel
      {
        T lm = T(0);
        bool lf = true;
#pragma omp for schedule(static) nowait
        for (long long i = 0; i < nc; ++i) {
          const T cs = sound_speed(P[i], P[(dim + 1) * nc + i], g);
          const T w = std::fabs(P[d * nc + i]) + cs;
          lm = lf ? w : jmax(lm, w);
          lf = false;
        }
#pragma omp critical
        {
          if (!lf) {
            m = first ? lm : jmax(m, lm);
            first = false;
          }
        }
      }
      alpha = m;
    }
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nc; ++i) {
      const long long im = G.shift(i, ax, -1), ip = G.shift(i, ax, 1);
      for (int v = 0; v < NV; ++v) {
        const T* p = P + v * nc;
        const T bd = (p[i] - p[im]) / dxT, fd = (p[ip] - p[i]) / dxT;
        D[v * nc + i] = limited(bd, fd, c.limiter, eps3dx) * dxT / T(2);
      }
    }
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nc; ++i) {
      const long long im = G.shift(i, ax, -1);
      T qL[5], qR[5], f[5];
      for (int v = 0; v < NV; ++v) {
        qL[v] = P[v * nc + im] + D[v * nc + im];
        qR[v] = P[v * nc + i] - D[v * nc + i];
      }
      if (c.riemann == R_HLL) hll(qL, qR, d, g, dim, f);
      else if (c.riemann == R_HLLC) hllc(qL, qR, d, g, dim, f);
      else lax_friedrichs(qL, qR, d, g, dim, alpha, f);
      for (int v = 0; v < NV; ++v) F[v * nc + i] = f[v];
    }
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nc; ++i) {
      const long long ip = G.shift(i, ax, 1);
      for (int v = 0; v < NV; ++v) U[v * nc + i] = U[v * nc + i] + inv_dx * (F[v * nc + i] - F[v * nc + ip]) * dt;
    }
  }
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < nc; ++i) {
    T u[5], q[5];
    for (int v = 0; v < NV; ++v) u[v] = U[v * nc + i];
    cons_to_prim(u, q, g, dim);
    for (int v = 0; v < NV; ++v) out[v * nc + i] = q[v];
  }
}

// SSP-RK2 of the gas rows (evolve_state.py:419-488), in place.
template <typename T>
void rk2(const Cfg& c, const Geo& G, T* gas, T dt, std::vector<T>* bufs) {
  const int dim = c.dim, NV = dim + 2;
  const long long nc = G.nc;
  const T g = T(c.gamma);
  std::vector<T>& P1 = bufs[0];
  std::vector<T>& P2 = bufs[1];
  stage(c, G, gas, P1.data(), dt, bufs[2], bufs[3], bufs[4]);
  stage(c, G, P1.data(), P2.data(), dt, bufs[2], bufs[3], bufs[4]);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < nc; ++i) {
    T q0[5], q2[5], U0[5], U2[5], U[5], q[5];
    for (int v = 0; v < NV; ++v) { q0[v] = gas[v * nc + i]; q2[v] = P2[v * nc + i]; }
    prim_to_cons(q0, U0, g, dim);
    prim_to_cons(q2, U2, g, dim);
    for (int v = 0; v < NV; ++v) U[v] = T(0.5) * (U0[v] + U2[v]);
    cons_to_prim(U, q, g, dim);
    for (int v = 0; v < NV; ++v) gas[v * nc + i] = q[v];
  }
}

// ------------------------------------------------------------ magnetic update

// curl by central differences (_vector_maths.py:55-100): f[3][nc] -> out[3][nc]
template <typename T>
void curl(const Geo& G, const T* f, T* out, T dxT) {
  const long long nc = G.nc;
  const int dim = G.dim;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < nc; ++i) {
    auto dF = [&](int comp, int ax) {
      return T(0.5) * (f[comp * nc + G.shift(i, ax, 1)] - f[comp * nc + G.shift(i, ax, -1)]) / dxT;
    };
    if (dim == 2) {
      out[i] = T(0) + dF(2, 1);
      out[nc + i] = T(0) + (-dF(2, 0));
      out[2 * nc + i] = T(0) + (dF(1, 0) - dF(0, 1));
    } else {
      out[i] = T(0) + (dF(2, 1) - dF(1, 2));
      out[nc + i] = T(0) + (dF(0, 2) - dF(2, 0));
      out[2 * nc + i] = T(0) + (dF(1, 0) - dF(0, 1));
    }
  }
}

template <typename T>
inline void cross3(const T* a, const T* b, T* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

// _magnetic_field_update.py:37-242 on the gas rows `gas` and the field `B`
// (3 rows), in place; returns the fixed-point iterations after the first
// evaluation.
template <typename T>
int magnetic_update(const Cfg& c, const Geo& G, T* gas, T* B, T dt, std::vector<T>* m) {
  const int dim = c.dim;
  const long long nc = G.nc;
  const T dxT = T(c.dx);
  T* v0 = m[0].data();   // velocity (3 rows)
  T* Bk = m[1].data();   // iterate
  T* vk = m[2].data();
  T* Bn = m[3].data();   // next iterate
  T* vn = m[4].data();
  T* av = m[5].data();   // averaged fields
  T* aB = m[6].data();
  T* Ef = m[7].data();   // cross(b, v), then curl(b)
  T* C1 = m[8].data();   // curl(E)
  T* C2 = m[9].data();   // curl(b)
  const T* rho = gas;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < nc; ++i) {
    v0[i] = gas[nc + i];
    v0[nc + i] = gas[2 * nc + i];
    v0[2 * nc + i] = (dim == 3) ? gas[3 * nc + i] : T(0);
  }
  // phi(v, b): curl(b x v), (b x curl b) / rho; B' = B - dt phi1, v' = v - dt phi2
  auto evaluate = [&](const T* vb, const T* bb, T* Bo, T* vo) {
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nc; ++i) {
      T b[3] = {bb[i], bb[nc + i], bb[2 * nc + i]}, v[3] = {vb[i], vb[nc + i], vb[2 * nc + i]}, e[3];
      cross3(b, v, e);
      for (int k = 0; k < 3; ++k) Ef[k * nc + i] = e[k];
    }
    curl(G, Ef, C1, dxT);
    curl(G, bb, C2, dxT);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nc; ++i) {
      T b[3] = {bb[i], bb[nc + i], bb[2 * nc + i]}, cb[3] = {C2[i], C2[nc + i], C2[2 * nc + i]}, p2[3];
      cross3(b, cb, p2);
      for (int k = 0; k < 3; ++k) {
        Bo[k * nc + i] = B[k * nc + i] - dt * C1[k * nc + i];
        vo[k * nc + i] = v0[k * nc + i] - dt * (p2[k] / rho[i]);
      }
    }
  };
  // the first evaluation at (B0 + B) / 2 = B, (v0 + v) / 2 = v
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < 3 * nc; ++i) {
    aB[i] = (B[i] + B[i]) / T(2);
    av[i] = (v0[i] + v0[i]) / T(2);
    Bk[i] = B[i];
    vk[i] = v0[i];
  }
  evaluate(av, aB, Bn, vn);
  int it = 0;
  for (;;) {
    double change = 0.0;
    bool first = true;
#pragma omp parallel
    {
      T lb = T(0), lv = T(0);
      bool lf = true;
#pragma omp for schedule(static) nowait
      for (long long i = 0; i < nc; ++i) {
        T db[3], dv[3];
        for (int k = 0; k < 3; ++k) { db[k] = Bk[k * nc + i] - Bn[k * nc + i]; dv[k] = vk[k * nc + i] - vn[k * nc + i]; }
        const T nb = std::sqrt(db[0] * db[0] + db[1] * db[1] + db[2] * db[2]);
        const T nv = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
        lb = lf ? nb : jmax(lb, nb);
        lv = lf ? nv : jmax(lv, nv);
        lf = false;
      }
#pragma omp critical
      {
        if (!lf) {
          const double mb = (double)lb, mv = (double)lv;
          const double mm = (mb != mb) ? mb : ((mv != mv) ? mv : std::max(mb, mv));
          change = first ? mm : ((mm != mm) ? mm : ((change != change) ? change : std::max(change, mm)));
          first = false;
        }
      }
    }
    if (!((change > c.tol) && (it < 1000))) break;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < 3 * nc; ++i) {
      Bk[i] = Bn[i];
      vk[i] = vn[i];
      if (c.midpoint) {
        aB[i] = (Bk[i] + B[i]) / T(2);
        av[i] = (vk[i] + v0[i]) / T(2);
      } else {
        aB[i] = Bk[i];
        av[i] = vk[i];
      }
    }
    evaluate(av, aB, Bn, vn);
    ++it;
  }
  // write-back with gamma = 5/3 (the refresh keeps p when |v| is unchanged)
  const T g53m1 = T(5.0 / 3.0 - 1.0);
  const T g53 = T(5.0 / 3.0);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < nc; ++i) {
    const T r = rho[i];
    const T va = std::sqrt(v0[i] * v0[i] + v0[nc + i] * v0[nc + i] + v0[2 * nc + i] * v0[2 * nc + i]);
    const T vb = std::sqrt(vn[i] * vn[i] + vn[nc + i] * vn[nc + i] + vn[2 * nc + i] * vn[2 * nc + i]);
    const T pold = gas[(dim + 1) * nc + i];
    T E = pold / g53m1 + T(0.5) * r * (va * va);
    E = E - T(0.5) * r * (va * va) + T(0.5) * r * (vb * vb);
    const T e = E / r - T(0.5) * (vb * vb);
    (void)g53;
    gas[(dim + 1) * nc + i] = g53m1 * r * e;
    for (int k = 0; k < dim; ++k) gas[(1 + k) * nc + i] = vn[k * nc + i];
    for (int k = 0; k < 3; ++k) B[k * nc + i] = Bn[k * nc + i];
  }
  return it;
}

// ------------------------------------------------------------ time loop

template <typename T>
double cfl_dt(const Cfg& c, const Geo& G, const T* P) {  // _timestep_estimator.py:95-128 (unsplit)
  const int dim = c.dim;
  const long long nc = G.nc;
  const T g = T(c.gamma);
  T m[3] = {T(0), T(0), T(0)};
  bool first = true;
#pragma omp parallel
  {
    T lm[3] = {T(0), T(0), T(0)};
    bool lf = true;
#pragma omp for schedule(static) nowait
    for (long long i = 0; i < nc; ++i) {
      const T cs = sound_speed(P[i], P[(dim + 1) * nc + i], g);
      for (int k = 0; k < dim; ++k) {
        const T w = std::fabs(P[(1 + k) * nc + i]) + cs;
        lm[k] = lf ? w : jmax(lm[k], w);
      }
      lf = false;
    }
#pragma omp critical
    {
      if (!lf) {
        for (int k = 0; k < dim; ++k) m[k] = first ? lm[k] : jmax(m[k], lm[k]);
        first = false;
      }
    }
  }
  const T dxT = T(c.dx);
  T total = m[0] / dxT;
  for (int k = 1; k < dim; ++k) total = total + m[k] / dxT;
  return (double)(T(c.C_cfl) * T(1) / total);
}

template <typename T>
int run(const Cfg& c, T* state, int64_t max_steps, double* t_out, int64_t* steps_out, int64_t* iters_out) {
  Geo G;
  G.init(c.dim, c.n);
  const long long nc = G.nc;
  const int NV = c.dim + 2;
  std::vector<T> bufs[5];
  bufs[0].assign((size_t)NV * nc, T(0));
  bufs[1].assign((size_t)NV * nc, T(0));
  bufs[2].assign((size_t)NV * nc, T(0));
  bufs[3].assign((size_t)NV * nc, T(0));
  bufs[4].assign((size_t)NV * nc, T(0));
  std::vector<T> mag[10];
  if (c.mhd)
    for (auto& v : mag) v.assign((size_t)3 * nc, T(0));
  double t = 0.0;
  int64_t steps = 0, iters = 0;
  while (steps < max_steps && t < c.t_end) {
    double dt = cfl_dt<T>(c, G, state);
    if (c.exact_end_time) dt = std::min(dt, c.t_end - t);
    const T dtT = T(dt);
    if (!c.mhd) {
      rk2(c, G, state, dtT, bufs);
    } else {
      T* gas = state;
      T* B = state + (size_t)NV * nc;
      rk2(c, G, gas, dtT / T(2), bufs);
      iters += magnetic_update(c, G, gas, B, dtT, mag);
      rk2(c, G, gas, dtT / T(2), bufs);
    }
    t = t + dt;
    ++steps;
  }
  *t_out = t;
  *steps_out = steps;
  *iters_out = iters;
  return 0;
}

}  // namespace

extern "C" {

// Runs at most max_steps adaptive FV steps of `state` (nv x n^dim values of
// dtype 0 = float32 / 1 = float64) in place, stopping at t_end.  limiter:
// 0 MINMOD, 1 OSHER, 2 DOUBLE_MINMOD, 3 SUPERBEE, 4 VAN_ALBADA; riemann: 0
// HLL, 1 HLLC, 3 Lax-Friedrichs; tol: the fixed-point tolerance.
// nthreads > 0 sets the OpenMP threads.  Returns 0, or 1 on bad arguments.
int amxref_fv_run(int dtype, int dim, int n, int mhd, int limiter, int riemann, int midpoint, double dx,
                  double gamma, double C_cfl, double t_end, double tol, int exact_end_time, int64_t max_steps,
                  void* state, double* t_out, int64_t* steps_out, int64_t* iters_out, int nthreads) {
  if ((dim != 2 && dim != 3) || n < 4 || !state || !t_out || !steps_out || !iters_out) return 1;
  if (limiter < 0 || limiter > 4 || (riemann != R_HLL && riemann != R_HLLC && riemann != R_LF)) return 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  Cfg c{dim, n, limiter, riemann, mhd, midpoint, dx, gamma, C_cfl, t_end, tol, exact_end_time};
  if (dtype == 0) return run<float>(c, static_cast<float*>(state), max_steps, t_out, steps_out, iters_out);
  return run<double>(c, static_cast<double*>(state), max_steps, t_out, steps_out, iters_out);
}

}  // extern "C"
