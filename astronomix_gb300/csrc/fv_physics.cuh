// Pointwise physics of the finite-volume Euler/MHD step, in registers.
//
// Every function restates one reference function with the same operand
// order, so that the FP64 instantiation reproduces the reference's FP64
// results to round-off and the FP32 instantiation mirrors its FP32 mode:
//
//   cons/prim/flux  astronomix/_fluid_equations/_equations.py:24-280,
//                   astronomix/_fluid_equations/_fluxes.py:25-93
//   limiters        astronomix/_finite_volume/_state_evolution/limiters.py:14-64,
//                   limited_gradients.py:22-88
//   HLL / HLLC      astronomix/_finite_volume/_riemann_solver/hll.py:36-261
//   Lax-Friedrichs  astronomix/_finite_volume/_riemann_solver/_lax_friedrichs.py:21-78
//
// A primitive vector of NV = DIM + 2 entries is (rho, v_1..v_DIM, p); the
// conserved one is (rho, m_1..m_DIM, E).  `d` is the 1-based flux axis.
#pragma once

#include <cuda_runtime.h>

namespace amx {

template <typename T> struct Num;
template <> struct Num<float> {
  static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
  static __device__ __forceinline__ float sin_(float x) { return sinf(x); }
  static __device__ __forceinline__ float abs_(float x) { return fabsf(x); }
};
template <> struct Num<double> {
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
  static __device__ __forceinline__ double sin_(double x) { return sin(x); }
  static __device__ __forceinline__ double abs_(double x) { return fabs(x); }
};

template <typename T> __device__ __forceinline__ T sq(T x) { return x * x; }

// jnp.sign
template <typename T> __device__ __forceinline__ T sgn(T x) {
  return x > T(0) ? T(1) : (x < T(0) ? T(-1) : (x == x ? T(0) : x));
}
// jnp.minimum / jnp.maximum (NaN-propagating)
template <typename T> __device__ __forceinline__ T jmin(T a, T b) {
  return (a != a) ? a : ((b != b) ? b : (b < a ? b : a));
}
template <typename T> __device__ __forceinline__ T jmax(T a, T b) {
  return (a != a) ? a : ((b != b) ? b : (b > a ? b : a));
}

// get_absolute_velocity (_equations.py:165-199)
template <typename T, int DIM>
__device__ __forceinline__ T abs_velocity(const T* q) {
  if (DIM == 1) return Num<T>::abs_(q[1]);
  if (DIM == 2) return Num<T>::sqrt_(q[1] * q[1] + q[2] * q[2]);
  return Num<T>::sqrt_(q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + T(1e-20));
}

// total_energy_from_primitives (_equations.py:253-266)
template <typename T>
__device__ __forceinline__ T total_energy(T rho, T u, T p, T gamma) {
  return p / (gamma - T(1)) + T(0.5) * rho * (u * u);
}

// pressure_from_energy (_equations.py:203-248)
template <typename T>
__device__ __forceinline__ T pressure_from_energy(T E, T rho, T u, T gamma) {
  const T e = E / rho - T(0.5) * (u * u);
  return (gamma - T(1)) * rho * e;
}

// conserved_state_from_primitive (_equations.py:104-156)
template <typename T, int DIM>
__device__ __forceinline__ void prim_to_cons(const T* q, T* U, T gamma) {
  const T rho = q[0];
  const T u = abs_velocity<T, DIM>(q);
  U[0] = rho;
#pragma unroll
  for (int a = 1; a <= DIM; ++a) U[a] = rho * q[a];
  U[DIM + 1] = total_energy(rho, u, q[DIM + 1], gamma);
}

// primitive_state_from_conserved (_equations.py:24-94)
template <typename T, int DIM>
__device__ __forceinline__ void cons_to_prim(const T* U, T* q, T gamma) {
  const T rho = U[0];
  const T E = U[DIM + 1];
  q[0] = rho;
  T u;
  if (DIM == 1) {
    q[1] = U[1] / rho;
    u = q[1];
  } else {
    T s = T(0);
#pragma unroll
    for (int a = 1; a <= DIM; ++a) {
      q[a] = U[a] / rho;
      s = (a == 1) ? q[a] * q[a] : s + q[a] * q[a];
    }
    u = Num<T>::sqrt_(s + T(1e-20));
  }
  q[DIM + 1] = pressure_from_energy(E, rho, u, gamma);
}

// _euler_flux (_fluxes.py:25-93)
template <typename T, int DIM>
__device__ __forceinline__ void euler_flux(const T* q, int d, T gamma, T* F) {
  const T rho = q[0], p = q[DIM + 1];
  const T ud = q[d];
  const T E = total_energy(rho, abs_velocity<T, DIM>(q), p, gamma);
  F[0] = ud * rho;
#pragma unroll
  for (int a = 1; a <= DIM; ++a) F[a] = ud * (q[a] * rho);
  F[DIM + 1] = ud * (p + E);
  F[d] = F[d] + p;
}

// speed_of_sound (_equations.py:269-280)
template <typename T>
__device__ __forceinline__ T sound_speed(T rho, T p, T gamma) {
  return Num<T>::sqrt_(gamma * p / rho);
}

// ------------------------------------------------------------ limiters

template <typename T> __device__ __forceinline__ T minmod(T a, T b) {
  return T(0.5) * (sgn(a) + sgn(b)) * jmin(Num<T>::abs_(a), Num<T>::abs_(b));
}
template <typename T> __device__ __forceinline__ T maxmod(T a, T b) {
  return T(0.5) * (sgn(a) + sgn(b)) * jmax(Num<T>::abs_(a), Num<T>::abs_(b));
}
template <typename T> __device__ __forceinline__ T minmod3(T a, T b, T c) {
  const bool same = (sgn(a) == sgn(b)) && (sgn(b) == sgn(c));
  return same ? sgn(a) * jmin(Num<T>::abs_(a), jmin(Num<T>::abs_(b), Num<T>::abs_(c))) : T(0);
}

// minmod(a, b) by cases: the smaller magnitude when a and b share a sign,
// else 0 -- equal to the sign formula for every finite input (a NaN gives 0
// here; the cell's own NaN still reaches its interface states)
template <typename T> __device__ __forceinline__ T minmod_cases(T a, T b) {
  return (a > T(0) && b > T(0)) ? (b < a ? b : a) : ((a < T(0) && b < T(0)) ? (b > a ? b : a) : T(0));
}

// The limited slope times dx / 2 of a cell from its neighbours, as the
// reconstruction adds it to the interface states: the reference's
// limited((q0 - qm) / dx, (qp - q0) / dx) dx / 2 (limited_gradients.py:22-88,
// reconstruction.py:399-431).  FP32 with MINMOD takes minmod(q0 - qm,
// qp - q0) / 2 directly: the same value up to the rounding of the two
// divisions and the product by dx, with no division.
template <typename T>
__device__ __forceinline__ T half_slope(T qm, T q0, T qp, int limiter, T dx);

// limited gradient from the backward/forward differences (already / dx)
template <typename T>
__device__ __forceinline__ T limited(T bd, T fd, int limiter, T dx) {
  switch (limiter) {
    case 0:  // MINMOD
      return minmod(bd, fd);
    case 1: {  // OSHER
      const T eps = T(1e-11);
      const T g = (Num<T>::abs_(bd) > eps) ? fd / (bd + eps) : T(0);
      return jmax(T(0), jmin(T(1.3), g)) * bd;
    }
    case 2:  // DOUBLE_MINMOD
      return (bd * fd > T(0)) ? minmod3((bd + fd) / T(2), T(2) * bd, T(2) * fd) : T(0);
    case 3:  // SUPERBEE
      return (bd * fd > T(0)) ? minmod(maxmod(bd, fd), minmod(T(2) * bd, T(2) * fd)) : T(0);
    default: {  // VAN_ALBADA
      const T eps = T(3) * dx;
      return ((fd * fd + eps) * bd + (bd * bd + eps) * fd) / (fd * fd + bd * bd + T(2) * eps);
    }
  }
}

template <typename T>
__device__ __forceinline__ T half_slope(T qm, T q0, T qp, int limiter, T dx) {
  if constexpr (sizeof(T) == 4) {
    if (limiter == 0) return minmod_cases(q0 - qm, qp - q0) * T(0.5);
  }
  return limited((q0 - qm) / dx, (qp - q0) / dx, limiter, dx) * dx / T(2);
}

// ------------------------------------------------------------ Riemann solvers

// RS_AM: the HLLC family with the compression switch of AM_HLLC /
// HYBRID_HLLC (FVArgs::am), a kernel of its own so that plain HLLC carries
// none of its code
enum { RS_HLL = 0, RS_HLLC = 1, RS_HLLC_LM = 2, RS_LF = 3, RS_AM = 4 };

// HLL (hll.py:36-109)
template <typename T, int DIM>
__device__ __forceinline__ void hll_flux(const T* qL, const T* qR, int d, T gamma, T* F) {
  constexpr int NV = DIM + 2;
  const T cL = sound_speed(qL[0], qL[NV - 1], gamma);
  const T cR = sound_speed(qR[0], qR[NV - 1], gamma);
  const T uL = qL[d], uR = qR[d];
  T FL[NV], FR[NV], UL[NV], UR[NV];
  euler_flux<T, DIM>(qL, d, gamma, FL);
  euler_flux<T, DIM>(qR, d, gamma, FR);
  const T SR = jmax(jmax(uL + cL, uR + cR), T(0));
  const T SL = jmin(jmin(uL - cL, uR - cR), T(0));
  prim_to_cons<T, DIM>(qL, UL, gamma);
  prim_to_cons<T, DIM>(qR, UR, gamma);
  const T SLSR = SL * SR;
  const T den = SR - SL;
#pragma unroll
  for (int v = 0; v < NV; ++v) F[v] = (SR * FL[v] - SL * FR[v] + SLSR * (UR[v] - UL[v])) / den;
}

// HLLC and HLLC-LM (hll.py:123-261); `lmdc`: the low-Mach dissipation
// control of AM_HLLC (:230-254), the velocity rows of the dissipation scaled
// by min(1, max |v| / c of the two states)
template <typename T, int DIM>
__device__ __forceinline__ void hllc_flux(const T* qL, const T* qR, int d, T gamma, bool lm, T* F,
                                          bool lmdc = false) {
  constexpr int NV = DIM + 2;
  const T rhoL = qL[0], rhoR = qR[0], pL = qL[NV - 1], pR = qR[NV - 1];
  const T uL = qL[d], uR = qR[d];
  const T cL = sound_speed(rhoL, pL, gamma);
  const T cR = sound_speed(rhoR, pR, gamma);
  T FL[NV], FR[NV], UL[NV], UR[NV];
  euler_flux<T, DIM>(qL, d, gamma, FL);
  euler_flux<T, DIM>(qR, d, gamma, FR);
  const T sL = Num<T>::sqrt_(rhoL), sR = Num<T>::sqrt_(rhoR);
  const T ssum = sL + sR;
  const T u_hat = (sL * uL + sR * uR) / ssum;
  const T c_hat_sq = (cL * cL * sL + cR * cR * sR) / ssum + T(0.5) * (sL * sR / (ssum * ssum)) * sq(uR - uL);
  const T c_hat = Num<T>::sqrt_(c_hat_sq);
  const T SL = jmin(uL - cL, u_hat - c_hat);
  const T SR = jmax(uR + cR, u_hat + c_hat);
  const T S_star = (pR - pL + rhoL * uL * (SL - uL) - rhoR * uR * (SR - uR)) /
                   (rhoL * (SL - uL) - rhoR * (SR - uR));
  prim_to_cons<T, DIM>(qL, UL, gamma);
  prim_to_cons<T, DIM>(qR, UR, gamma);
  T USL[NV], USR[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) { USL[v] = UL[v]; USR[v] = UR[v]; }
  USL[d] = rhoL * S_star;
  USL[NV - 1] = USL[NV - 1] + (S_star - uL) * (rhoL * S_star + pL / (SL - uL));
  USR[d] = rhoR * S_star;
  USR[NV - 1] = USR[NV - 1] + (S_star - uR) * (rhoR * S_star + pR / (SR - uR));
  const T fL = SL - uL, gL = SL - S_star, fR = SR - uR, gR = SR - S_star;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    USL[v] = USL[v] * fL / gL;
    USR[v] = USR[v] * fR / gR;
  }
  T SLs = SL, SRs = SR;
  if (lm) {
    const T Ma = jmax(Num<T>::abs_(uL / cL), Num<T>::abs_(uR / cR));
    const T phi = Num<T>::sin_(jmin(T(1), Ma / T(0.1)) * T(3.141592653589793) / T(2));
    SLs = SL * phi;
    SRs = SR * phi;
  }
  const T aS = Num<T>::abs_(S_star);
  T fm = T(1);
  if (lmdc) {
    const T Ma = jmax(Num<T>::abs_(abs_velocity<T, DIM>(qL) / cL), Num<T>::abs_(abs_velocity<T, DIM>(qR) / cR));
    fm = jmin(T(1), Ma);
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    T Fs;
    if (lmdc && v >= 1 && v <= DIM)
      Fs = T(0.5) * (FL[v] + FR[v]) +
           fm * (T(0.5) * (SLs * (USL[v] - UL[v]) + aS * (USL[v] - USR[v]) + SRs * (USR[v] - UR[v])));
    else
      Fs = T(0.5) * (FL[v] + FR[v]) +
           T(0.5) * (SLs * (USL[v] - UL[v]) + aS * (USL[v] - USR[v]) + SRs * (USR[v] - UR[v]));
    T f = (SL >= T(0)) ? FL[v] : Fs;
    F[v] = (SR <= T(0)) ? FR[v] : f;
  }
}

// The compression switch of AM_HLLC / HYBRID_HLLC (hll.py:268-326) at a
// cell of a primitive tile: div v by central differences (each axis
// (v[+1] - v[-1]) / 2dx, summed in axis order) below -0.05 c / dx.
// `q` points at the cell's density in a tile whose variable rows are
// `vstride` apart; stride[a] is the cell stride along axis a.
template <typename T, int DIM>
__device__ __forceinline__ bool am_compressed(const T* q, int vstride, const int* stride, T gamma, T dx) {
  T div = T(0);
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    const T* v = q + (1 + a) * vstride;
    div = div + (v[stride[a]] - v[-stride[a]]) / (T(2) * dx);
  }
  const T c = sound_speed(q[0], q[(DIM + 1) * vstride], gamma);
  return div < T(-0.05) * c / dx;
}

// Lax-Friedrichs with the global alpha of the stage (_lax_friedrichs.py:21-78)
template <typename T, int DIM>
__device__ __forceinline__ void lf_flux(const T* qL, const T* qR, int d, T gamma, T alpha, T* F) {
  constexpr int NV = DIM + 2;
  T FL[NV], FR[NV], UL[NV], UR[NV];
  prim_to_cons<T, DIM>(qL, UL, gamma);
  prim_to_cons<T, DIM>(qR, UR, gamma);
  euler_flux<T, DIM>(qL, d, gamma, FL);
  euler_flux<T, DIM>(qR, d, gamma, FR);
  const T ha = T(0.5) * alpha;
#pragma unroll
  for (int v = 0; v < NV; ++v) F[v] = T(0.5) * (FL[v] + FR[v]) - ha * (UR[v] - UL[v]);
}

// `lm` selects the HLLC-LM variant inside the HLLC family and `lmdc` the
// low-Mach dissipation control (runtime flags)
template <typename T, int DIM, int RS>
__device__ __forceinline__ void riemann(const T* qL, const T* qR, int d, T gamma, T alpha, bool lm, T* F,
                                        bool lmdc = false) {
  if (RS == RS_HLL) hll_flux<T, DIM>(qL, qR, d, gamma, F);
  else if (RS == RS_HLLC) hllc_flux<T, DIM>(qL, qR, d, gamma, lm, F);
  else if (RS == RS_AM) hllc_flux<T, DIM>(qL, qR, d, gamma, lm, F, lmdc);
  else if (RS == RS_HLLC_LM) hllc_flux<T, DIM>(qL, qR, d, gamma, true, F);
  else lf_flux<T, DIM>(qL, qR, d, gamma, alpha, F);
}

}  // namespace amx
