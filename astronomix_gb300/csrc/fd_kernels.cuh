// Finite-difference WENO-CT MHD step (3D, periodic): device code.
//
// Restates astronomix/_finite_difference/** (leo1200/astronomix 0.5.1):
//
//   cons/prim, floors      _fluid_equations/_equations.py:135-222,
//                          _enforce_positivity.py:24-59
//   MHD x-flux             _fluid_equations/_fluxes.py:23-69
//   eigensystem            _fluid_equations/_eigen.py:28-993
//   WENO flux              _interface_fluxes/_weno.py:112-324
//   CT                     _magnetic_update/_constrained_transport.py:44-198
//   maths                  _maths/_interpolate.py, _maths/_differencing.py
//   SSPRK(5,4) with CT     _time_integrators/_ssprk.py:178-347
//   CFL                    _timestep_estimation/_timestep_estimator.py:26-91
//
// GB300 design: the reference recomputes the whole eigensystem 14 times per
// direction per stage and makes full transposed copies for the y and z
// fluxes; here each interface computes its eigenvector blocks once from
// per-cell quantities staged in shared memory, the y/z fluxes run in place
// with a component permutation, and the stencil chains of CT are separate
// sweeps whose intermediates stay in HBM/L2.
//
// Conserved rows: rho, mx, my, mz, E, Bx, By, Bz; primitive state rows 0-7 the
// same with velocities / pressure, rows 8-10 the face fields bx, by, bz
// (index i of a face array holds the face i+1/2).
#pragma once

#include "amx_common.cuh"
#include "fv_physics.cuh"

namespace amx {
namespace fd {

enum { RHO = 0, MX = 1, MY = 2, MZ = 3, EN = 4, BX = 5, BY = 6, BZ = 7 };

// ---------------------------------------------------------------- control

struct FDControl {
  unsigned long long lam[4];   // bitwise maxima of |lambda| per direction
  double dt;
  double t;
  long long steps;
  int active;                  // 1 while the current step runs
  int status;
  unsigned int done_count;     // last-block counter of the CFL reduction
  unsigned int pad0;
};

struct FDArgs {
  int n;
  long long nc;
  double dx;
  double gamma;
  double rhomin, pgmin;
  double C_cfl, dt_max, t_end;
  int enforce_positivity;
  int exact_end_time;
  int fixed_timestep;
  double dt_fixed;
  double t_pause;
  // stellar wind EI source (stellar_wind.py:485-584); wind = 0: none
  int wind;
  double wind_mdot;    // mass-loss rate
  double wind_vinf;    // final velocity
  double wind_V;       // sum of the injection mask x dx^3 (computed on the host)
  double wind_rinj;    // injection radius, num_injection_cells dx
  double wind_r1;      // 1.3 x the injection radius (end of the taper)
  double box;          // box size (cell radii from the box centre)
  int wind_lo;         // the cube of cells that holds the taper: [wind_lo, wind_lo + wind_n) per axis
  int wind_n;
};

// kernels of a step, for the per-kernel timing of amx_plan_profile
enum FDPhase {
  FD_PH_CFL = 0, FD_PH_PREP, FD_PH_WENO_X, FD_PH_WENO_Y, FD_PH_WENO_Z, FD_PH_EMF, FD_PH_EMF_AVG, FD_PH_WIND,
  FD_PH_UPDATE, FD_PH_FINALIZE, FD_PH_FORCING, FD_PH_ADVANCE, FD_PH_COUNT
};
constexpr int kFDMaxMarks = 48;  // launches of one step (38, 43 with the wind source, 44 with forcing)

// buffers and launch geometry handed from the host plan to the typed launchers
struct FDLaunch {
  int grid;        // blocks of the pointwise sweeps
  int n;
  void* bufs[10];  // Q0 Q QF QC (8 rows) ACC (16) B BF (3) M (6) OM OB (3)
  FDControl* ctl;
  void* wind_src;  // stellar wind: [5][wind_n^3] source of the current stage (null without)
  // per-kernel timing (null when off): an event is recorded after every
  // launch, and marks_kind[i] names the kernel that ends at marks[i]
  cudaEvent_t* marks;
  int* marks_kind;
  int* marks_used;
};

// records the end of a launch of kind `k` (no-op when timing is off)
inline void fd_mark(const FDLaunch& L, int k, cudaStream_t s) {
  if (!L.marks || *L.marks_used >= kFDMaxMarks) return;
  L.marks_kind[*L.marks_used] = k;
  cudaEventRecord(L.marks[*L.marks_used], s);
  ++*L.marks_used;
}

int fd_set_attrs_f32();
int fd_set_attrs_f64();
int fd_launch_stages_f32(const FDLaunch& L, void* state, const FDArgs& a, cudaStream_t s);
int fd_launch_stages_f64(const FDLaunch& L, void* state, const FDArgs& a, cudaStream_t s);
int fd_launch_cfl_f32(const FDLaunch& L, const void* state, const FDArgs& a, cudaStream_t s);
int fd_launch_cfl_f64(const FDLaunch& L, const void* state, const FDArgs& a, cudaStream_t s);

// ---------------------------------------------------------------- indexing

__device__ __forceinline__ long long cidx(int i, int j, int k, int n) {
  return ((long long)i * n + j) * n + k;
}

// neighbour of cell c along axis ax (0 = x, 1 = y, 2 = z) with periodic wrap
__device__ __forceinline__ long long nb(int i, int j, int k, int ax, int off, int n) {
  if (ax == 0) i = wrap(i + off, n);
  else if (ax == 1) j = wrap(j + off, n);
  else k = wrap(k + off, n);
  return cidx(i, j, k, n);
}

__device__ __forceinline__ void decompose(long long c, int n, int* i, int* j, int* k) {
  *k = (int)(c % n);
  *j = (int)((c / n) % n);
  *i = (int)(c / ((long long)n * n));
}

// ---------------------------------------------------------------- equations

// conserved_state_from_primitive_mhd (_equations.py:135-170)
template <typename T>
__device__ __forceinline__ void prim_to_cons(const T* P, T* U, T gamma) {
  const T rho = P[RHO];
  const T u2 = P[MX] * P[MX] + P[MY] * P[MY] + P[MZ] * P[MZ];
  const T b2 = P[BX] * P[BX] + P[BY] * P[BY] + P[BZ] * P[BZ];
  U[RHO] = rho;
  U[MX] = rho * P[MX];
  U[MY] = rho * P[MY];
  U[MZ] = rho * P[MZ];
  U[EN] = P[EN] / (gamma - T(1)) + T(0.5) * rho * u2 + T(0.5) * b2;
  U[BX] = P[BX];
  U[BY] = P[BY];
  U[BZ] = P[BZ];
}

// primitive_state_from_conserved_mhd (_equations.py:174-222)
template <typename T>
__device__ __forceinline__ void cons_to_prim(const T* U, T* P, T gamma, T rhomin, T pgmin, bool floors) {
  const T rho = U[RHO];
  const T ux = U[MX] / rho, uy = U[MY] / rho, uz = U[MZ] / rho;
  const T u2 = ux * ux + uy * uy + uz * uz;
  const T b2 = U[BX] * U[BX] + U[BY] * U[BY] + U[BZ] * U[BZ];
  T p = (gamma - T(1)) * (U[EN] - T(0.5) * rho * u2 - T(0.5) * b2);
  P[RHO] = rho;
  P[MX] = ux;
  P[MY] = uy;
  P[MZ] = uz;
  P[BX] = U[BX];
  P[BY] = U[BY];
  P[BZ] = U[BZ];
  if (floors) {
    P[RHO] = jmax(rho, rhomin);
    p = jmax(p, pgmin);
  }
  P[EN] = p;
}

// _enforce_positivity (_enforce_positivity.py:24-59): rho and E in place
template <typename T>
__device__ __forceinline__ void positivity(T* U, T gamma, T rhomin, T pgmin) {
  const T rho = jmax(U[RHO], rhomin);
  const T vx = U[MX] / rho, vy = U[MY] / rho, vz = U[MZ] / rho;
  const T b2 = U[BX] * U[BX] + U[BY] * U[BY] + U[BZ] * U[BZ];
  const T v2 = vx * vx + vy * vy + vz * vz;
  T p = (gamma - T(1)) * (U[EN] - T(0.5) * rho * v2 - T(0.5) * b2);
  p = jmax(p, pgmin);
  U[EN] = p / (gamma - T(1)) + T(0.5) * rho * v2 + T(0.5) * b2;
  U[RHO] = rho;
}

// _mhd_flux_x (_fluxes.py:23-69), on a state already permuted so that the
// flux direction is "x"
template <typename T>
__device__ __forceinline__ void mhd_flux(const T* U, T* F, T gamma, T rhomin, T pgmin, bool floors) {
  T P[8];
  cons_to_prim(U, P, gamma, rhomin, pgmin, floors);
  const T rho = P[RHO], vx = P[MX], vy = P[MY], vz = P[MZ];
  const T Bx = P[BX], By = P[BY], Bz = P[BZ], p = P[EN];
  const T b2 = Bx * Bx + By * By + Bz * Bz;
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T ptot = p + T(0.5) * b2;
  const T vdotB = vx * Bx + vy * By + vz * Bz;
  const T E = p / (gamma - T(1)) + T(0.5) * rho * v2 + T(0.5) * b2;
  F[RHO] = rho * vx;
  F[MX] = rho * (vx * vx) + ptot - Bx * Bx;
  F[MY] = rho * vx * vy - Bx * By;
  F[MZ] = rho * vx * vz - Bx * Bz;
  F[EN] = (E + ptot) * vx - vdotB * Bx;
  F[BX] = T(0);
  F[BY] = By * vx - Bx * vy;
  F[BZ] = Bz * vx - Bx * vz;
}

template <typename T>
__device__ __forceinline__ T dss(T x) {  // diff_safe_sqrt (_eigen.py:21-24)
  return Num<T>::sqrt_(jmax(x, T(1e-12)));
}

// _eigenvalue_building_blocks (_eigen.py:28-114) of one cell: vx, cf, ca, cs
template <typename T>
__device__ __forceinline__ void eigenvalue_blocks(const T* U, T gamma, T rhomin, T pgmin, T* vx_, T* cf_,
                                                  T* ca_, T* cs_) {
  T rho = U[RHO];
  const T vx = U[MX] / rho, vy = U[MY] / rho, vz = U[MZ] / rho;
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T Bx = U[BX], By = U[BY], Bz = U[BZ];
  const T b2 = Bx * Bx + By * By + Bz * Bz;
  T pg = (gamma - T(1)) * (U[EN] - T(0.5) * (rho * v2 + b2));
  rho = ((rho < rhomin) || (pg < pgmin)) ? jmax(rho, rhomin) : rho;
  pg = ((rho < rhomin) || (pg < pgmin)) ? jmax(pg, pgmin) : pg;
  const T cs2 = jmax(T(0), gamma * Num<T>::abs_(pg / rho));
  const T b2r = b2 / rho;
  const T disc = dss(jmax(T(0), sq(b2r + cs2) - T(4) * (Bx * Bx) / rho * cs2));
  *vx_ = vx;
  *cf_ = dss(jmax(T(0), T(0.5) * (b2r + cs2 + disc)));
  *ca_ = dss(jmax(T(0), (Bx * Bx) / rho));
  *cs_ = dss(jmax(T(0), T(0.5) * (b2r + cs2 - disc)));
}

// per-cell inputs of the eigenvector blocks (_eigen.py:124-162): floored rho,
// velocities (from the unfloored rho), specific enthalpy
template <typename T>
__device__ __forceinline__ void eigvec_cell(const T* U, T gamma, T rhomin, T pgmin, T* out /*rho,vx,vy,vz,h*/) {
  T rho = U[RHO];
  const T vx = U[MX] / rho, vy = U[MY] / rho, vz = U[MZ] / rho;
  const T vsq = vx * vx + vy * vy + vz * vz;
  const T Bx = U[BX], By = U[BY], Bz = U[BZ];
  const T bsq = Bx * Bx + By * By + Bz * Bz;
  T energy = U[EN];
  T pg = (gamma - T(1)) * (energy - T(0.5) * (rho * vsq + bsq));
  rho = ((rho < rhomin) || (pg < pgmin)) ? jmax(rho, rhomin) : rho;
  pg = ((rho < rhomin) || (pg < pgmin)) ? jmax(pg, pgmin) : pg;
  energy = ((rho < rhomin) || (pg < pgmin)) ? pg / (gamma - T(1)) + T(0.5) * (rho * vsq + bsq) : energy;
  out[0] = rho;
  out[1] = vx;
  out[2] = vy;
  out[3] = vz;
  out[4] = (energy + pg) / rho;
}

// interface eigenvector blocks (_eigen.py:164-337)
template <typename T>
struct EigIF {
  T vx, vy, vz, vsq, by, bz, bty, btz, sbx, sbt, a, a2, a2inv, cf, cs, af, as, sr, gam0, gam1, gam2;
  bool ge;
};

template <typename T>
__device__ __forceinline__ void eig_interface(const T* cL, const T* cR, T BxL, T ByL, T BzL, T BxR, T ByR, T BzR,
                                              T gamma, EigIF<T>& e) {
  const T r = T(0.5) * (cL[0] + cR[0]);
  const T vx = T(0.5) * (cL[1] + cR[1]);
  const T vy = T(0.5) * (cL[2] + cR[2]);
  const T vz = T(0.5) * (cL[3] + cR[3]);
  const T bx = T(0.5) * (BxL + BxR);
  const T by = T(0.5) * (ByL + ByR);
  const T bz = T(0.5) * (BzL + BzR);
  const T h = T(0.5) * (cL[4] + cR[4]);
  const T vsq = vx * vx + vy * vy + vz * vz;
  const T bsq = bx * bx + by * by + bz * bz;
  const T b2r = bsq / r;
  const T bx2r = (bx * bx) / r;
  const T a2 = (gamma - T(1)) * (h - T(0.5) * (vsq + b2r));
  const T a = dss(jmax(T(0), a2));
  const T disc = sq(b2r + a2) - T(4) * bx2r * a2;
  const T disc_r = dss(jmax(T(0), disc));
  const T cf = dss(jmax(T(0), T(0.5) * (b2r + a2 + disc_r)));
  const T ca = dss(jmax(T(0), bx2r));
  const T cs = dss(jmax(T(0), T(0.5) * (b2r + a2 - disc_r)));
  T bt2 = by * by + bz * bz;
  const T sbx = (bx >= T(0)) ? T(1) : T(-1);
  bt2 = jmax(bt2, T(1e-12));
  const T bty = (bt2 >= T(1e-12)) ? by / dss(bt2) : T(1) / dss(T(2));
  const T btz = (bt2 >= T(1e-12)) ? bz / dss(bt2) : T(1) / dss(T(2));
  T denom = cf * cf - cs * cs;
  denom = jmax(denom, T(1e-12));
  const T af = (denom >= T(1e-12)) ? dss(jmax(T(0), a2 - cs * cs)) / dss(denom) : T(1);
  const T as = (denom >= T(1e-12)) ? dss(jmax(T(0), cf * cf - a2)) / dss(denom) : T(1);
  e.vx = vx;
  e.vy = vy;
  e.vz = vz;
  e.vsq = vsq;
  e.by = by;
  e.bz = bz;
  e.bty = bty;
  e.btz = btz;
  e.sbx = sbx;
  e.sbt = (by != T(0)) ? ((by >= T(0)) ? T(1) : T(-1)) : ((bz >= T(0)) ? T(1) : T(-1));
  e.a = a;
  e.a2 = a2;
  e.a2inv = (a2 > T(0)) ? T(1) / a2 : T(0);
  e.cf = cf;
  e.cs = cs;
  e.af = af;
  e.as = as;
  e.sr = dss(r);
  e.gam0 = T(1) - gamma;
  e.gam1 = T(0.5) * (gamma - T(1));
  e.gam2 = (gamma - T(2)) / (gamma - T(1));
  e.ge = a >= ca;
}

// left eigenvector row s (_eigen.py:677-909)
template <typename T>
__device__ __forceinline__ void L_row(const EigIF<T>& e, int s, T* L) {
  const T vx = e.vx, vy = e.vy, vz = e.vz, vsq = e.vsq, bty = e.bty, btz = e.btz, sbx = e.sbx;
  const T a = e.a, cf = e.cf, cs = e.cs, af = e.af, aS = e.as, sr = e.sr;
  const T gam0 = e.gam0, gam1 = e.gam1;
#pragma unroll
  for (int k = 0; k < 8; ++k) L[k] = T(0);
  switch (s) {
    case 0:
    case 6: {
      if (s == 0) {  // fast -
        L[RHO] = af * (gam1 * vsq + cf * vx) - aS * cs * (bty * vy + btz * vz) * sbx;
        L[MX] = af * (gam0 * vx - cf);
        L[MY] = gam0 * af * vy + aS * cs * bty * sbx;
        L[MZ] = gam0 * af * vz + aS * cs * btz * sbx;
      } else {  // fast +
        L[RHO] = af * (gam1 * vsq - cf * vx) + aS * cs * (bty * vy + btz * vz) * sbx;
        L[MX] = af * (gam0 * vx + cf);
        L[MY] = gam0 * af * vy - aS * cs * bty * sbx;
        L[MZ] = gam0 * af * vz - aS * cs * btz * sbx;
      }
      L[BY] = gam0 * af * e.by + a * aS * bty * sr;
      L[BZ] = gam0 * af * e.bz + a * aS * btz * sr;
      L[EN] = -gam0 * af;
#pragma unroll
      for (int k = 0; k < 8; ++k) L[k] = T(0.5) * L[k] * e.a2inv;
      if (!e.ge) {
#pragma unroll
        for (int k = 0; k < 8; ++k) L[k] = L[k] * e.sbt;
      }
      break;
    }
    case 1:
    case 5: {
      L[RHO] = btz * vy - bty * vz;
      L[MY] = -btz;
      L[MZ] = bty;
      if (s == 1) {
        L[BY] = -btz * sbx * sr;
        L[BZ] = bty * sbx * sr;
      } else {
        L[BY] = btz * sbx * sr;
        L[BZ] = -bty * sbx * sr;
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) L[k] = T(0.5) * L[k];
      break;
    }
    case 2:
    case 4: {
      if (s == 2) {
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
#pragma unroll
      for (int k = 0; k < 8; ++k) L[k] = T(0.5) * L[k] * e.a2inv;
      if (e.ge) {
#pragma unroll
        for (int k = 0; k < 8; ++k) L[k] = L[k] * e.sbt;
      }
      break;
    }
    default: {  // 3: entropy
      L[RHO] = -e.a2 / gam0 - T(0.5) * vsq;
      L[MX] = vx;
      L[MY] = vy;
      L[MZ] = vz;
      L[BY] = e.by;
      L[BZ] = e.bz;
      L[EN] = T(-1);
#pragma unroll
      for (int k = 0; k < 8; ++k) L[k] = -gam0 * L[k] * e.a2inv;
      break;
    }
  }
}

// right eigenvector column s (_eigen.py:392-620)
template <typename T>
__device__ __forceinline__ void R_col(const EigIF<T>& e, int s, T* R) {
  const T vx = e.vx, vy = e.vy, vz = e.vz, vsq = e.vsq, bty = e.bty, btz = e.btz, sbx = e.sbx;
  const T a = e.a, a2 = e.a2, cf = e.cf, cs = e.cs, af = e.af, aS = e.as, sr = e.sr, gam2 = e.gam2;
#pragma unroll
  for (int k = 0; k < 8; ++k) R[k] = T(0);
  switch (s) {
    case 0:
      R[RHO] = af;
      R[MX] = af * (vx - cf);
      R[MY] = af * vy + aS * cs * bty * sbx;
      R[MZ] = af * vz + aS * cs * btz * sbx;
      R[BY] = a * aS * bty / sr;
      R[BZ] = a * aS * btz / sr;
      R[EN] = af * (cf * cf - cf * vx + T(0.5) * vsq - gam2 * a2) + aS * cs * (bty * vy + btz * vz) * sbx;
      break;
    case 1:
      R[MY] = -btz;
      R[MZ] = bty;
      R[BY] = -btz * sbx / sr;
      R[BZ] = bty * sbx / sr;
      R[EN] = bty * vz - btz * vy;
      break;
    case 2:
      R[RHO] = aS;
      R[MX] = aS * (vx - cs);
      R[MY] = aS * vy - af * cf * bty * sbx;
      R[MZ] = aS * vz - af * cf * btz * sbx;
      R[BY] = -a * af * bty / sr;
      R[BZ] = -a * af * btz / sr;
      R[EN] = aS * (cs * cs - cs * vx + T(0.5) * vsq - gam2 * a2) - af * cf * (bty * vy + btz * vz) * sbx;
      break;
    case 3:
      R[RHO] = T(1);
      R[MX] = vx;
      R[MY] = vy;
      R[MZ] = vz;
      R[EN] = T(0.5) * vsq;
      break;
    case 4:
      R[RHO] = aS;
      R[MX] = aS * (vx + cs);
      R[MY] = aS * vy + af * cf * bty * sbx;
      R[MZ] = aS * vz + af * cf * btz * sbx;
      R[BY] = -a * af * bty / sr;
      R[BZ] = -a * af * btz / sr;
      R[EN] = aS * (cs * cs + cs * vx + T(0.5) * vsq - gam2 * a2) + af * cf * (bty * vy + btz * vz) * sbx;
      break;
    case 5:
      R[MY] = -btz;
      R[MZ] = bty;
      R[BY] = btz * sbx / sr;
      R[BZ] = -bty * sbx / sr;
      R[EN] = bty * vz - btz * vy;
      break;
    default:  // 6
      R[RHO] = af;
      R[MX] = af * (vx + cf);
      R[MY] = af * vy - aS * cs * bty * sbx;
      R[MZ] = af * vz - aS * cs * btz * sbx;
      R[BY] = a * aS * bty / sr;
      R[BZ] = a * aS * btz / sr;
      R[EN] = af * (cf * cf + cf * vx + T(0.5) * vsq - gam2 * a2) - aS * cs * (bty * vy + btz * vz) * sbx;
      break;
  }
  const bool flip = (s == 0 || s == 6) ? !e.ge : ((s == 2 || s == 4) ? e.ge : false);
  if (flip) {
#pragma unroll
    for (int k = 0; k < 8; ++k) R[k] = R[k] * e.sbt;
  }
}

// Max for the WENO flux where a NaN operand needs no propagation of its own:
// any NaN in a stencil cell already reaches the flux through the
// projections, so the flux is NaN either way.  One min/max instruction in
// FP32; the NaN-propagating jmax in FP64, whose arithmetic stays the
// reference's.
template <typename T>
__device__ __forceinline__ T wmax(T a, T b) {
  if constexpr (sizeof(T) == 4) return fmaxf(a, b);
  else return jmax(a, b);
}

// WENO interpolant of _weno.py:190-205 / 213-228.  FP32: one reciprocal of
// the weight sum and products with 1/3, 1/6 in place of four divisions (the
// FP32 kernels are held to an L1 tolerance against FP64); FP64: the
// reference's divisions.
template <typename T>
__device__ __forceinline__ T weno_phi(T a, T b, T c, T d) {
  const T eps = T(1e-8);
  const T IS0 = T(13) * sq(a - b) + T(3) * sq(a - T(3) * b);
  const T IS1 = T(13) * sq(b - c) + T(3) * sq(b + c);
  const T IS2 = T(13) * sq(c - d) + T(3) * sq(T(3) * c - d);
  const T al0 = T(1) / sq(eps + IS0);
  const T al1 = T(6) / sq(eps + IS1);
  const T al2 = T(3) / sq(eps + IS2);
  T asum = al0 + al1 + al2;
  asum = wmax(asum, T(1e-14));
  if constexpr (sizeof(T) == 4) {
    const T r = T(1) / asum;
    return (al0 * r) * (a - T(2) * b + c) * T(1.0 / 3.0) + (al2 * r - T(0.5)) * (b - T(2) * c + d) * T(1.0 / 6.0);
  } else {
    const T w0 = al0 / asum;
    const T w2 = al2 / asum;
    return w0 * (a - T(2) * b + c) / T(3) + (w2 - T(0.5)) * (b - T(2) * c + d) / T(6);
  }
}

// interp_center_to_face (_interpolate.py:9-21): (-f[-1] + 9 f[0] + 9 f[1] - f[2]) / 16
template <typename T>
__device__ __forceinline__ T c2f(T m1, T p0, T p1, T p2) {
  return (-m1 + T(9) * p0 + T(9) * p1 - p2) / T(16);
}

// interp_face_to_center (_interpolate.py:24-36) from faces i-3 .. i+2
template <typename T>
__device__ __forceinline__ T f2c(T m3, T m2, T m1, T p0, T p1, T p2) {
  return (T(3) * m3 - T(25) * m2 + T(150) * m1 + T(150) * p0 - T(25) * p1 + T(3) * p2) / T(256);
}

// finite_difference_int6 (_differencing.py:9-30) from faces i-3 .. i+2
template <typename T>
__device__ __forceinline__ T fd6(T m3, T m2, T m1, T p0, T p1, T p2) {
  const T c1 = T(75.0 / 64.0), c2 = T(-25.0 / 384.0), c3 = T(3.0 / 640.0);
  return c1 * (p0 - m1) + c2 * (p1 - m2) + c3 * (p2 - m3);
}

// the component permutation that makes axis `d` the "x" of _weno_flux_x:
// identity for x, swap x<->y for y, swap x<->z for z (_weno.py:244-324)
__device__ __forceinline__ int perm_row(int d, int row) {
  if (d == 1) {
    if (row == MX) return MY;
    if (row == MY) return MX;
    if (row == BX) return BY;
    if (row == BY) return BX;
  } else if (d == 2) {
    if (row == MX) return MZ;
    if (row == MZ) return MX;
    if (row == BX) return BZ;
    if (row == BZ) return BX;
  }
  return row;
}

// the same permutation, usable in constant expressions
__host__ __device__ constexpr int perm_row_c(int d, int row) {
  return d == 1   ? (row == MX ? MY : row == MY ? MX : row == BX ? BY : row == BY ? BX : row)
         : d == 2 ? (row == MX ? MZ : row == MZ ? MX : row == BX ? BZ : row == BZ ? BX : row)
                  : row;
}

}  // namespace fd
}  // namespace amx
