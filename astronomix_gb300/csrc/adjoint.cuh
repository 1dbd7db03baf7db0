// Discrete adjoint of the finite-volume MHD step (reverse mode, by hand).
//
// The forward step (fv_kernels.cuh) is
//
//   S1 = L(S0, h)                 stage 1, h = dt/2 (dt without MHD)
//   S2 = C(S0, L(S1, h))          stage 2 with the RK2 combination
//   Z0 = G(B0, v0), Z(j+1) = G(Zj)    fixed-point evaluations of the magnetic map
//   S3 = W(S2, Zk)                write-back (pressure refresh)
//   S4 = L(S3, h), S5 = C(S3, L(S4, h))
//
// with L(P, h) = prim(cons(P) + h/dx sum_axes (F[i-1/2] - F[i+1/2])),
// C(P0, P) = prim((cons(P0) + cons(P)) / 2) (evolve_state.py:339-488) and G
// the implicit-midpoint map of _magnetic_field_update.py:82-165.  Its
// vector-Jacobian products, derived by hand, run as stream-ordered kernels
// over a tape of S0..S4 and the iterates Zj that a forward replay records
// with the forward's own dt and iteration count (dt is not differentiated:
// time_integration.py:632-661 wraps it in stop_gradient; the fixed point is
// differentiated through the iterations it took, like reverse mode through
// the reference's while loop).
//
// Derivative conventions follow JAX (and torch.autograd): d|x| = sign(x) dx
// with sign(0) = 0, d sign = 0, and min/max split the cotangent equally on
// ties.  Two compositions that are the identity in exact arithmetic are
// differentiated as the identity: cons(prim(U)) inside the RK2 combination
// and the gamma = 5/3 pressure refresh (p_new = p when the kinetic energy is
// removed and added back; _magnetic_field_update.py:208-222).  Where the
// reference evaluates |v| as a square root of zero (the refresh at v = 0),
// reverse mode through it gives NaN; the identity gives the finite limit.
//
// Scope: periodic boundaries, MINMOD limiter, HLL fluxes, implicit midpoint
// or implicit Euler magnetic integrator, 2D and 3D.
#pragma once

#include "fv_kernels.cuh"

namespace amx {
namespace adj {

constexpr int kThreads = 256;

// ------------------------------------------------------------ scalar rules

// d jmax(x, y): weight of x (ties split equally)
template <typename T> __device__ __forceinline__ T wmax(T x, T y) {
  return x > y ? T(1) : (x == y ? T(0.5) : T(0));
}
template <typename T> __device__ __forceinline__ T wmin(T x, T y) {
  return x < y ? T(1) : (x == y ? T(0.5) : T(0));
}

// partial derivatives of minmod(a, b) = (sign a + sign b)/2 * min(|a|, |b|)
template <typename T>
__device__ __forceinline__ void minmod_d(T a, T b, T* ga, T* gb) {
  const T s = T(0.5) * (sgn(a) + sgn(b));
  const T aa = Num<T>::abs_(a), ab = Num<T>::abs_(b);
  const T wa = wmin(aa, ab), wb = wmin(ab, aa);
  *ga = s * wa * sgn(a);
  *gb = s * wb * sgn(b);
}

// |v|^2 as the forward forms it (abs_velocity squared); FP32 skips the
// square root and its square (the same value up to rounding)
template <typename T, int DIM>
__device__ __forceinline__ T vsq(const T* q) {
  if constexpr (sizeof(T) == 4 && DIM >= 2) {
    T s = q[1] * q[1] + q[2] * q[2];
    if (DIM == 3) s = s + q[3] * q[3] + T(1e-20);
    return s;
  }
  const T u = abs_velocity<T, DIM>(q);
  return u * u;
}

// the wave-speed bounds' maxima and minima: NaN-propagating in FP64 as the
// forward's, plain min/max instructions in FP32 (a NaN state has no
// gradient worth keeping)
template <typename T> __device__ __forceinline__ T vmax(T a, T b) {
  if constexpr (sizeof(T) == 4) return fmaxf(a, b);
  else return jmax(a, b);
}
template <typename T> __device__ __forceinline__ T vmin(T a, T b) {
  if constexpr (sizeof(T) == 4) return fminf(a, b);
  else return jmin(a, b);
}

// ------------------------------------------------------------ pointwise VJPs

// lq += (dU/dq)^T lU for U = prim_to_cons(q)
template <typename T, int DIM>
__device__ __forceinline__ void prim_to_cons_vjp(const T* q, const T* lU, T gamma, T* lq) {
  constexpr int E = DIM + 1;
  const T rho = q[0];
  T r = lU[0] + lU[E] * T(0.5) * vsq<T, DIM>(q);
#pragma unroll
  for (int a = 1; a <= DIM; ++a) {
    r += lU[a] * q[a];
    lq[a] += lU[a] * rho + lU[E] * rho * q[a];
  }
  lq[0] += r;
  lq[E] += lU[E] / (gamma - T(1));
}

// lU = (dq/dU)^T lq for q = cons_to_prim(U)
template <typename T, int DIM>
__device__ __forceinline__ void cons_to_prim_vjp(const T* U, const T* lq, T gamma, T* lU) {
  constexpr int E = DIM + 1;
  const T rho = U[0];
  T q[DIM + 2];
  cons_to_prim<T, DIM>(U, q, gamma);
  // p = (gamma - 1) rho e, e = E / rho - |v|^2 / 2
  const T e = U[E] / rho - T(0.5) * vsq<T, DIM>(q);
  const T le = lq[E] * (gamma - T(1)) * rho;
  T lrho = lq[0] + lq[E] * (gamma - T(1)) * e - le * U[E] / (rho * rho);
  lU[E] = le / rho;
#pragma unroll
  for (int a = 1; a <= DIM; ++a) {
    const T lv = lq[a] - le * q[a];  // |v|^2 enters e with -1/2
    lU[a] = lv / rho;
    lrho -= lv * q[a] / rho;
  }
  lU[0] = lrho;
}

// lq += (dF/dq)^T lF for F = euler_flux(q, d)
template <typename T, int DIM>
__device__ __forceinline__ void euler_flux_vjp(const T* q, int d, T gamma, const T* lF, T* lq) {
  constexpr int E = DIM + 1;
  const T rho = q[0], p = q[E], ud = q[d];
  const T v2 = vsq<T, DIM>(q);
  const T En = total_energy(rho, abs_velocity<T, DIM>(q), p, gamma);
  T lrho = lF[0] * ud + lF[E] * ud * T(0.5) * v2;
  T lud = lF[0] * rho + lF[E] * (p + En);
#pragma unroll
  for (int a = 1; a <= DIM; ++a) {
    lrho += lF[a] * ud * q[a];
    lud += lF[a] * q[a] * rho;
    lq[a] += lF[a] * ud * rho + lF[E] * ud * rho * q[a];
  }
  lq[0] += lrho;
  lq[d] += lud;
  lq[E] += lF[d] + lF[E] * ud * (T(1) + T(1) / (gamma - T(1)));
}

// (lqL, lqR) += VJP of the HLL flux (hll.py:36-109)
template <typename T, int DIM>
__device__ __forceinline__ void hll_vjp(const T* qL, const T* qR, int d, T gamma, const T* lF, T* lqL, T* lqR) {
  constexpr int NV = DIM + 2, E = DIM + 1;
  const T rhoL = qL[0], rhoR = qR[0], pL = qL[E], pR = qR[E];
  const T uL = qL[d], uR = qR[d];
  const T cL = sound_speed(rhoL, pL, gamma), cR = sound_speed(rhoR, pR, gamma);
  T FL[NV], FR[NV], UL[NV], UR[NV];
  euler_flux<T, DIM>(qL, d, gamma, FL);
  euler_flux<T, DIM>(qR, d, gamma, FR);
  prim_to_cons<T, DIM>(qL, UL, gamma);
  prim_to_cons<T, DIM>(qR, UR, gamma);
  const T a1 = uL + cL, a2 = uR + cR, b1 = uL - cL, b2 = uR - cR;
  const T ma = vmax(a1, a2), mb = vmin(b1, b2);
  const T SR = vmax(ma, T(0)), SL = vmin(mb, T(0));
  const T rden = T(1) / (SR - SL);
  T lnum[NV], lFL[NV], lFR[NV], lUL[NV], lUR[NV];
  T lden = T(0), lSR = T(0), lSL = T(0);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const T num = SR * FL[v] - SL * FR[v] + SL * SR * (UR[v] - UL[v]);
    lnum[v] = lF[v] * rden;
    lden -= lnum[v] * num * rden;
    lFL[v] = SR * lnum[v];
    lFR[v] = -SL * lnum[v];
    lUR[v] = SL * SR * lnum[v];
    lUL[v] = -lUR[v];
    lSR += lnum[v] * (FL[v] + SL * (UR[v] - UL[v]));
    lSL += lnum[v] * (-FR[v] + SR * (UR[v] - UL[v]));
  }
  lSR += lden;
  lSL -= lden;
  // SR = max(max(a1, a2), 0), SL = min(min(b1, b2), 0)
  const T lma = lSR * wmax(ma, T(0)), lmb = lSL * wmin(mb, T(0));
  const T la1 = lma * wmax(a1, a2), la2 = lma * wmax(a2, a1);
  const T lb1 = lmb * wmin(b1, b2), lb2 = lmb * wmin(b2, b1);
  const T lcL = la1 - lb1, lcR = la2 - lb2;
  lqL[d] += la1 + lb1;
  lqR[d] += la2 + lb2;
  // c = sqrt(gamma p / rho)
  const T rrL = T(1) / rhoL, rrR = T(1) / rhoR;
  const T kL = lcL * (T(0.5) * gamma) * rrL / cL, kR = lcR * (T(0.5) * gamma) * rrR / cR;
  lqL[E] += kL;
  lqL[0] -= kL * pL * rrL;
  lqR[E] += kR;
  lqR[0] -= kR * pR * rrR;
  euler_flux_vjp<T, DIM>(qL, d, gamma, lFL, lqL);
  euler_flux_vjp<T, DIM>(qR, d, gamma, lFR, lqR);
  prim_to_cons_vjp<T, DIM>(qL, lUL, gamma, lqL);
  prim_to_cons_vjp<T, DIM>(qR, lUR, gamma, lqR);
}

// ------------------------------------------------------------ kernels

template <typename T>
struct AdjGrid {
  int n;
  long long nc;
  double dx;
  double inv_dx;  // 1 / dx (computed on the host)
  double gamma;
};

template <int DIM>
__device__ __forceinline__ void decompose(long long c, int n, int* ic) {
  if (DIM == 2) { ic[0] = (int)(c / n); ic[1] = (int)(c % n); ic[2] = 0; }
  else { ic[2] = (int)(c % n); ic[1] = (int)((c / n) % n); ic[0] = (int)(c / ((long long)n * n)); }
}

template <int DIM>
__device__ __forceinline__ long long shifted(const int* ic, int k, int off, int n) {
  int j[3] = {ic[0], ic[1], ic[2]};
  j[k] = wrap(j[k] + off, n);
  return cell_index<DIM>(j[0], j[1], j[2], n);
}

// Line tiles of the flux adjoint along axis K: L = 32 cells along K by W = 8
// lines along J (the contiguous axis when K is not, else the next-to-last
// axis); the halo of a line costs 3 + 3 cells of 32.
//
// Shared memory per line: P (PL cells), lU and the limited slope D
// (UL cells each), the cotangents of qL and qR (FL faces each) and, in FP32,
// the two partial derivatives of the limiter (UL cells each); FP64 recomputes
// those in the cell phase so that two blocks still fit on an SM.
template <int DIM, int K>
struct AxisTile {
  static constexpr bool KFAST = (K == DIM - 1);
  static constexpr int L = 32;
  static constexpr int W = 8;
  static constexpr int J = KFAST ? DIM - 2 : DIM - 1;
  static constexpr int M = 3 - K - J;  // third axis (3D only)
  static constexpr int PL = L + 6, UL = L + 4, FL = L + 3;
  static constexpr int LP = L + 1;  // pitch of the staged lPin of the tile's cells (odd)
  // one thread per face and per cell: every phase but the halo load runs in
  // a single round
  static constexpr int THREADS = W * (L + 4);
  template <typename T>
  static constexpr bool keep_partials() { return sizeof(T) == 4; }
  // FIRST (the pass that also does the stage's pointwise part) stages the
  // stage output and its cotangent (UL cells), P0 and lP0 (the tile's cells)
  template <typename T, bool FIRST>
  static constexpr size_t smem(int nv) {
    return sizeof(T) * (size_t)nv * W *
           (PL + 2 * UL + 2 * FL + (keep_partials<T>() ? 2 * UL : 0) + LP + (FIRST ? 2 * UL + 2 * LP : 0));
  }
};

// The flux terms of one axis: for every face f (between cells f-1 and f) of
// the tile and its reach, the cotangent of the HLL flux
// lF = dt/dx (lU[f] - lU[f-1]) is pulled back through the flux and the
// limited reconstruction qL = P[f-1] + D[f-1], qR = P[f] - D[f],
// D[m] = minmod((P[m] - P[m-1]) / dx, (P[m+1] - P[m]) / dx) dx / 2
// (reconstruction.py:399-431, limited_gradients.py:22-88), and every cell of
// the tile gathers the faces that read it (f in [m-1, m+2]) into lPin.
//
// FIRST (the pass along the contiguous axis, which runs first) also does the
// pointwise part of the stage: it forms lU from the stage output (P_out =
// prim(U), or with P0 the RK2 combination prim((cons(P0) + cons(prim(U)))/2),
// whose cons(prim(.)) is differentiated as the identity) on its line
// segments, writes lU for the other passes, adds the P0 term into lP0 and
// sets (or, with `accumulate`, adds) lPin = (d cons(P_in))^T lU + its own
// flux terms.  The other passes add their flux terms to lPin.
template <typename T, int DIM, int K, bool FIRST>
__global__ void __launch_bounds__(AxisTile<DIM, K>::THREADS, sizeof(T) == 4 ? 3 : 2)
k_stage_axis(AdjGrid<T> g, const T* Pin, const T* Pout, const T* P0, const T* lPout, T* lU, T* lPin, T* lP0,
             int accumulate, T h) {
  using A = AxisTile<DIM, K>;
  constexpr int NV = DIM + 2, L = A::L, W = A::W;
  constexpr bool KEEP = A::template keep_partials<T>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sP = reinterpret_cast<T*>(smem_raw);   // [NV][W][PL], cell m at m + 3
  T* sU = sP + NV * W * A::PL;              // [NV][W][UL], cell m at m + 2
  T* sD = sU + NV * W * A::UL;              // [NV][W][UL] limited slope, cell m at m + 2
  T* sLL = sD + NV * W * A::UL;             // [NV][W][FL] cotangent of qL, face f at f + 1
  T* sLR = sLL + NV * W * A::FL;
  T* sGa = sLR + NV * W * A::FL;            // [NV][W][UL] d minmod / d backward difference (FP32)
  T* sGb = sGa + NV * W * A::UL;            // d minmod / d forward difference
  // [NV][W][LP] lPin of the tile's cells, after the partials in FP32 and in
  // their place in FP64; then (FIRST) P_out, lP_out [NV][W][UL] and P0, lP0
  // [NV][W][LP]
  T* sLin = KEEP ? sGb + NV * W * A::UL : sGa;
  T* sQo = sLin + NV * W * A::LP;
  T* sLo = sQo + NV * W * A::UL;
  T* sP0 = sLo + NV * W * A::UL;
  T* sLP0 = sP0 + NV * W * A::LP;
  const int n = g.n;
  const long long nc = g.nc;
  const T gamma = T(g.gamma);
  const T dxT = T(g.dx);
  const T inv_dx = T(g.inv_dx);

  // tile origin
  const int tK = (n + L - 1) / L, tJ = (n + W - 1) / W;
  long long b = blockIdx.x;
  const int bK = (int)(b % tK);
  b /= tK;
  const int bJ = (int)(b % tJ);
  b /= tJ;
  const int oK = bK * L, oJ = bJ * W, oM = (DIM == 3) ? (int)b : 0;

  auto cell = [&](int l, int w) -> long long {  // l may be outside [0, L): periodic along K
    int x = oK + l;
    while (x < 0) x += n;
    while (x >= n) x -= n;
    int ic[3] = {0, 0, 0};
    ic[K] = x;
    ic[A::J] = oJ + w;
    if (DIM == 3) ic[A::M] = oM;
    return cell_index<DIM>(ic[0], ic[1], ic[2], n);
  };
  // element e of a [W][len] array: lines vary fastest when K is not the
  // contiguous axis (then the lines are contiguous in memory)
  auto split = [&](int e, int len, int* w, int* m) {
    if (A::KFAST) { *w = e / len; *m = e % len; } else { *w = e % W; *m = e / W; }
  };

  // loads: P for m in [-3, L+2], lU for m in [-2, L+1].  The copies go
  // straight to shared memory (cp.async), every one of a thread's issued
  // before it waits for any: the pass is bound by their latency otherwise.
  for (int e = threadIdx.x; e < W * A::PL; e += blockDim.x) {
    int w, m;
    split(e, A::PL, &w, &m);
    m -= 3;
    if (oJ + w >= n) continue;
    const long long c = cell(m, w);
#pragma unroll
    for (int v = 0; v < NV; ++v) cp_async_elem(sP + (v * W + w) * A::PL + m + 3, Pin + v * nc + c);
  }
  for (int e = threadIdx.x; e < W * A::UL; e += blockDim.x) {
    int w, m;
    split(e, A::UL, &w, &m);
    m -= 2;
    if (oJ + w >= n) continue;
    const long long c = cell(m, w);
    const int o = w * A::UL + m + 2;
    if (!FIRST) {
#pragma unroll
      for (int v = 0; v < NV; ++v) cp_async_elem(sU + v * W * A::UL + o, lU + v * nc + c);
    } else {
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        cp_async_elem(sQo + v * W * A::UL + o, Pout + v * nc + c);
        cp_async_elem(sLo + v * W * A::UL + o, lPout + v * nc + c);
      }
    }
  }
  const bool want_lin = !FIRST || accumulate;
  for (int e = threadIdx.x; e < W * L; e += blockDim.x) {
    int w, l;
    split(e, L, &w, &l);
    if (oJ + w >= n || oK + l >= n) continue;
    const long long c = cell(l, w);
    const int o = w * A::LP + l;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      if (want_lin) cp_async_elem(sLin + v * W * A::LP + o, lPin + v * nc + c);
      if (FIRST && P0) {
        cp_async_elem(sP0 + v * W * A::LP + o, P0 + v * nc + c);
        cp_async_elem(sLP0 + v * W * A::LP + o, lP0 + v * nc + c);
      }
    }
  }
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  // FIRST: lU of the cells m in [-2, L+1] from the stage output and its
  // cotangent (read by the face phase, after the next barrier)
  if (FIRST) {
    for (int e = threadIdx.x; e < W * A::UL; e += blockDim.x) {
      int w, m;
      split(e, A::UL, &w, &m);
      if (oJ + w >= n) continue;
      const int o = w * A::UL + m;
      T q[NV], U[NV], lq[NV], lu[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) { q[v] = sQo[v * W * A::UL + o]; lq[v] = sLo[v * W * A::UL + o]; }
      prim_to_cons<T, DIM>(q, U, gamma);
      cons_to_prim_vjp<T, DIM>(U, lq, gamma, lu);
      if (P0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) lu[v] = T(0.5) * lu[v];
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) sU[v * W * A::UL + o] = lu[v];
    }
  }
  // the limited slope D[m] = minmod(bd, fd) dx / 2 of every cell m in
  // [-2, L+1], once, as the forward's reconstruction forms it (FP32:
  // minmod of the differences by cases, /2; FP64: the reference's
  // formula), and in FP32 its partial derivatives
  for (int e = threadIdx.x; e < W * A::UL; e += blockDim.x) {
    int w, m;
    split(e, A::UL, &w, &m);
    if (oJ + w >= n) continue;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const T* sp = sP + (v * W + w) * A::PL + 1;  // cell m at sp[m]
      const int o = (v * W + w) * A::UL + m;
      sD[o] = half_slope(sp[m - 1], sp[m], sp[m + 1], 0, dxT);
      if (KEEP) {
        // d minmod / d(a, b) by cases: the smaller magnitude's weight (ties
        // split equally) where a and b share a sign, else 0
        const T a_ = sp[m] - sp[m - 1], b_ = sp[m + 1] - sp[m];
        const bool same = (a_ > T(0) && b_ > T(0)) || (a_ < T(0) && b_ < T(0));
        const T aa = Num<T>::abs_(a_), ab = Num<T>::abs_(b_);
        sGa[o] = same ? (aa < ab ? T(1) : (aa == ab ? T(0.5) : T(0))) : T(0);
        sGb[o] = same ? (ab < aa ? T(1) : (aa == ab ? T(0.5) : T(0))) : T(0);
      }
    }
  }
  __syncthreads();
  // faces f in [-1, L+1]: qL = P[f-1] + D[f-1], qR = P[f] - D[f]
  for (int e = threadIdx.x; e < W * A::FL; e += blockDim.x) {
    int w, f;
    split(e, A::FL, &w, &f);
    f -= 1;
    if (oJ + w >= n) continue;
    T qL[NV], qR[NV], lF[NV], lL[NV], lR[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const T* sp = sP + (v * W + w) * A::PL + 3;
      const T* d = sD + (v * W + w) * A::UL + 2;
      qL[v] = sp[f - 1] + d[f - 1];
      qR[v] = sp[f] - d[f];
      const T* u = sU + (v * W + w) * A::UL + 2;
      // U[i] += inv_dx (F[i-1/2] - F[i+1/2]) h: face f feeds cell f (+) and f - 1 (-)
      lF[v] = inv_dx * (u[f] - u[f - 1]) * h;
      lL[v] = T(0);
      lR[v] = T(0);
    }
    hll_vjp<T, DIM>(qL, qR, K + 1, gamma, lF, lL, lR);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      sLL[(v * W + w) * A::FL + f + 1] = lL[v];
      sLR[(v * W + w) * A::FL + f + 1] = lR[v];
    }
  }
  __syncthreads();
  // cells of the tile
  for (int e = threadIdx.x; e < W * L; e += blockDim.x) {
    int w, l;
    split(e, L, &w, &l);
    if (oJ + w >= n || oK + l >= n) continue;
    const long long c = cell(l, w);
    T r[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const T* LL = sLL + (v * W + w) * A::FL + 1;
      const T* LR = sLR + (v * W + w) * A::FL + 1;
      T ga0, gb0, gap, gbm;
      if (KEEP) {
        const int o = (v * W + w) * A::UL + 2 + l;
        ga0 = sGa[o];
        gb0 = sGb[o];
        gap = sGa[o + 1];
        gbm = sGb[o - 1];
      } else {
        const T* sp = sP + (v * W + w) * A::PL + 3;
        T t0, t1;
        minmod_d((sp[l] - sp[l - 1]) / dxT, (sp[l + 1] - sp[l]) / dxT, &ga0, &gb0);
        minmod_d((sp[l + 1] - sp[l]) / dxT, (sp[l + 2] - sp[l + 1]) / dxT, &gap, &t0);
        minmod_d((sp[l - 1] - sp[l - 2]) / dxT, (sp[l] - sp[l - 1]) / dxT, &t1, &gbm);
      }
      // cotangent of the slope D[m] = lqL[m+1] - lqR[m]
      const T dm1 = LL[l] - LR[l - 1], d0 = LL[l + 1] - LR[l], dp1 = LL[l + 2] - LR[l + 1];
      r[v] = LL[l + 1] + LR[l] + d0 * (ga0 - gb0) / T(2) - dp1 * gap / T(2) + dm1 * gbm / T(2);
    }
    if (FIRST) {
      T lu[NV], qi[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        lu[v] = sU[(v * W + w) * A::UL + l + 2];
        qi[v] = sP[(v * W + w) * A::PL + l + 3];
        lU[v * nc + c] = lu[v];
      }
      prim_to_cons_vjp<T, DIM>(qi, lu, gamma, r);
      if (P0) {
        T q0[NV], l0[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) { q0[v] = sP0[(v * W + w) * A::LP + l]; l0[v] = T(0); }
        prim_to_cons_vjp<T, DIM>(q0, lu, gamma, l0);
#pragma unroll
        for (int v = 0; v < NV; ++v) lP0[v * nc + c] = sLP0[(v * W + w) * A::LP + l] + l0[v];
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) lPin[v * nc + c] = accumulate ? sLin[(v * W + w) * A::LP + l] + r[v] : r[v];
    } else {
#pragma unroll
      for (int v = 0; v < NV; ++v) lPin[v * nc + c] = sLin[(v * W + w) * A::LP + l] + r[v];
    }
  }
}

// ---- magnetic map

// iterate (B, v) at cell c: from the iterate buffer, or (first evaluation)
// B0 and v0 (vz = 0 in 2D)
template <typename T, int DIM>
__device__ __forceinline__ void load_Z(const T* Z, const T* S, long long c, long long nc, T* B, T* v) {
  if (Z) {
#pragma unroll
    for (int i = 0; i < 3; ++i) { B[i] = Z[i * nc + c]; v[i] = Z[(3 + i) * nc + c]; }
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) B[i] = S[(DIM + 2 + i) * nc + c];
    v[0] = S[nc + c];
    v[1] = S[2 * nc + c];
    v[2] = (DIM == 3) ? S[3 * nc + c] : T(0);
  }
}

template <typename T, int DIM>
__device__ __forceinline__ void load_B0v0(const T* S, long long c, long long nc, T* B, T* v) {
  load_Z<T, DIM>(nullptr, S, c, nc, B, v);
}

// averaged fields at c (midpoint) or the iterate (Euler)
template <typename T, int DIM>
__device__ __forceinline__ void avg_at(const T* Z, const T* S, long long c, long long nc, bool midpoint, T* Ba,
                                       T* va) {
  T Bk[3], vk[3], B0[3], v0[3];
  load_Z<T, DIM>(Z, S, c, nc, Bk, vk);
  load_B0v0<T, DIM>(S, c, nc, B0, v0);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Ba[i] = midpoint ? (Bk[i] + B0[i]) / T(2) : Bk[i];
    va[i] = midpoint ? (vk[i] + v0[i]) / T(2) : vk[i];
  }
}

// curl by central differences of a 3-vector field given per neighbour
// (Fp[k] = F at c + e_k, Fm[k] = F at c - e_k), _vector_maths.py:55-100
template <typename T, int DIM>
__device__ __forceinline__ void curl_c(T (*Fp)[3], T (*Fm)[3], T dx, T* out) {
  auto D = [&](int i, int k) { return T(0.5) * (Fp[k][i] - Fm[k][i]) / dx; };
  if (DIM == 2) {
    out[0] = D(2, 1);
    out[1] = -D(2, 0);
    out[2] = D(1, 0) - D(0, 1);
  } else {
    out[0] = D(2, 1) - D(1, 2);
    out[1] = D(0, 2) - D(2, 0);
    out[2] = D(1, 0) - D(0, 1);
  }
}

// Pass 1 of the adjoint of one evaluation (B', v') = G(Z) with
// B' = B0 - h curl(Ba x va), v' = v0 - h (Ba x curl Ba) / rho:
//   lE = -h curl(lB')   (the central-difference curl is its own transpose
//                        on a periodic grid)
//   lX = -h lv' / rho,  lrho += h lv'.X / rho^2
//   lBa = va x lE + J x lX (+ curl(lJ) in pass 2), lva = lE x Ba, lJ = lX x Ba
// and lB0 += lB', lv0 += lv'.  Writes lJ, the partial lBa and lva.
// Tiles of the point-wise magnetic adjoint: 256 cells, halo 1.
template <int DIM> struct MagAdjTile;
template <> struct MagAdjTile<2> {
  static constexpr int T0 = 16, T1 = 16, T2 = 1;
};
template <> struct MagAdjTile<3> {
  static constexpr int T0 = 4, T1 = 8, T2 = 8;
};

// The averaged B (Ba) and the cotangent lB' of a halo-1 tile are staged in
// shared memory; each cell reads its neighbours' values there.
template <typename T, int DIM>
__global__ void __launch_bounds__(kThreads)
k_mag_adj1(AdjGrid<T> g, const T* Z, const T* S, const T* lZn, T h, int midpoint, T* lJ, T* lBa, T* lva,
           T* lB0, T* lv0, T* lrho) {
  using A = MagAdjTile<DIM>;
  constexpr int H0 = A::T0 + 2, H1 = A::T1 + 2, H2 = (DIM == 3) ? A::T2 + 2 : 1;
  constexpr int HALO = H0 * H1 * H2;
  __shared__ T sB[3][HALO];
  __shared__ T sL[3][HALO];
  const long long nc = g.nc;
  const int n = g.n;
  const T dx = T(g.dx);
  const int n0 = (n + A::T0 - 1) / A::T0, n1 = (n + A::T1 - 1) / A::T1;
  int b = blockIdx.x;
  const int o0 = (b % n0) * A::T0;
  b /= n0;
  const int o1 = (b % n1) * A::T1;
  b /= n1;
  const int o2 = (DIM == 3) ? b * A::T2 : 0;
  for (int e = threadIdx.x; e < HALO; e += blockDim.x) {
    const int e2 = e % H2, e1 = (e / H2) % H1, e0 = e / (H2 * H1);
    // periodic halo index (g >= -1): compares instead of two divisions a coordinate
    auto per = [n](int g) {
      if (g < 0) g += n;
      while (g >= n) g -= n;
      return g;
    };
    const int i0 = per(o0 + e0 - 1), i1 = per(o1 + e1 - 1);
    const int i2 = (DIM == 3) ? per(o2 + e2 - 1) : 0;
    const long long c = cell_index<DIM>(i0, i1, i2, n);
    T Ba[3], va[3];
    avg_at<T, DIM>(Z, S, c, nc, midpoint != 0, Ba, va);
#pragma unroll
    for (int i = 0; i < 3; ++i) { sB[i][e] = Ba[i]; sL[i][e] = lZn[i * nc + c]; }
  }
  __syncthreads();
  const int cl = threadIdx.x;  // one cell per thread
  const int c2 = (DIM == 3) ? cl % A::T2 : 0;
  const int c1 = (DIM == 3) ? (cl / A::T2) % A::T1 : cl % A::T1;
  const int c0 = (DIM == 3) ? cl / (A::T2 * A::T1) : cl / A::T1;
  const int g0 = o0 + c0, g1 = o1 + c1, g2 = o2 + c2;
  if (g0 >= n || g1 >= n || (DIM == 3 && g2 >= n)) return;
  const long long c = cell_index<DIM>(g0, g1, g2, n);
  const int hc = ((c0 + 1) * H1 + (c1 + 1)) * H2 + (DIM == 3 ? c2 + 1 : 0);
  const int st[3] = {H1 * H2, H2, 1};
  T Bp[3][3], Bm[3][3], Lp[3][3], Lm[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int i = 0; i < 3; ++i) Bp[k][i] = Bm[k][i] = Lp[k][i] = Lm[k][i] = T(0);
#pragma unroll
  for (int k = 0; k < DIM; ++k)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      Bp[k][i] = sB[i][hc + st[k]];
      Bm[k][i] = sB[i][hc - st[k]];
      Lp[k][i] = sL[i][hc + st[k]];
      Lm[k][i] = sL[i][hc - st[k]];
    }
  T Ba[3], va[3];
  avg_at<T, DIM>(Z, S, c, nc, midpoint != 0, Ba, va);
  T J[3], lE[3];
  curl_c<T, DIM>(Bp, Bm, dx, J);
  curl_c<T, DIM>(Lp, Lm, dx, lE);
#pragma unroll
  for (int i = 0; i < 3; ++i) lE[i] = -h * lE[i];
  T X[3];
  cross3(Ba, J, X);
  const T rho = S[c];
  T lX[3], lvn[3];
  T lr = T(0);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    lvn[i] = lZn[(3 + i) * nc + c];
    lX[i] = -h * lvn[i] / rho;
    lr += h * lvn[i] * X[i] / (rho * rho);
  }
  T t1[3], t2[3], lvA[3], lJc[3];
  cross3(va, lE, t1);
  cross3(J, lX, t2);
  cross3(lE, Ba, lvA);
  cross3(lX, Ba, lJc);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    lJ[i * nc + c] = lJc[i];
    lBa[i * nc + c] = t1[i] + t2[i];
    lva[i * nc + c] = lvA[i];
    lB0[i * nc + c] += sL[i][hc];
    lv0[i * nc + c] += lvn[i];
  }
  lrho[c] += lr;
}

template <typename T, int DIM>
unsigned mag_adj_blocks(int n) {
  using A = MagAdjTile<DIM>;
  long long b = (long long)((n + A::T0 - 1) / A::T0) * ((n + A::T1 - 1) / A::T1);
  if (DIM == 3) b *= (n + A::T2 - 1) / A::T2;
  return (unsigned)b;
}

// Pass 2: lBa += curl(lJ); then Ba = (Bk + B0)/2 (or Bk) hands lBa, lva to
// the iterate (lZ, or B0 / v0 for the first evaluation) and to B0 / v0.
template <typename T, int DIM>
__global__ void __launch_bounds__(kThreads)
k_mag_adj2(AdjGrid<T> g, const T* lJ, const T* lBa, const T* lva, int midpoint, int first, T* lZ, T* lB0,
           T* lv0, T* lS2) {
  const long long nc = g.nc;
  const int n = g.n;
  const T dx = T(g.dx);
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (long long)gridDim.x * blockDim.x) {
    int ic[3];
    decompose<DIM>(c, n, ic);
    T Lp[3][3], Lm[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int i = 0; i < 3; ++i) Lp[k][i] = Lm[k][i] = T(0);
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const long long cp = shifted<DIM>(ic, k, +1, n), cm = shifted<DIM>(ic, k, -1, n);
#pragma unroll
      for (int i = 0; i < 3; ++i) { Lp[k][i] = lJ[i * nc + cp]; Lm[k][i] = lJ[i * nc + cm]; }
    }
    T cJ[3];
    curl_c<T, DIM>(Lp, Lm, dx, cJ);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T lb = lBa[i * nc + c] + cJ[i];
      const T lv = lva[i * nc + c];
      const T bk = midpoint ? lb / T(2) : lb, vk = midpoint ? lv / T(2) : lv;
      const T b0 = midpoint ? lb / T(2) : T(0), v0 = midpoint ? lv / T(2) : T(0);
      if (first) {
        // the last pass: v0 is the gas velocity of S2 (its z row is the
        // synthesised vz = 0 in 2D)
        lB0[i * nc + c] += bk + b0;
        const T lv = lv0[i * nc + c] + vk + v0;
        if (i < DIM) lS2[(1 + i) * nc + c] += lv;
      } else {
        lZ[i * nc + c] = bk;
        lZ[(3 + i) * nc + c] = vk;
        lB0[i * nc + c] += b0;
        lv0[i * nc + c] += v0;
      }
    }
  }
}

// Adjoint of the write-back S3 = W(S2, Z) (_magnetic_field_update.py:208-242):
// rho and p pass through (the refresh is the identity on p), the velocity
// and B rows of S3 come from the final iterate Z.  Sets lS2's density and
// pressure rows and zeroes its velocity and B rows (they accumulate the
// magnetic iterations' cotangents of v0 and B0); sets lZ.
template <typename T, int DIM>
__global__ void __launch_bounds__(kThreads)
k_final_adj(AdjGrid<T> g, const T* lS3, T* lZ, T* lS2, T* lv0) {
  const long long nc = g.nc;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (long long)gridDim.x * blockDim.x) {
    lS2[c] = lS3[c];
    lS2[(DIM + 1) * nc + c] = lS3[(DIM + 1) * nc + c];
#pragma unroll
    for (int i = 0; i < DIM; ++i) lS2[(1 + i) * nc + c] = T(0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      lS2[(DIM + 2 + i) * nc + c] = T(0);
      lZ[i * nc + c] = lS3[(DIM + 2 + i) * nc + c];
      lZ[(3 + i) * nc + c] = (i < DIM) ? lS3[(1 + i) * nc + c] : T(0);
      lv0[i * nc + c] = T(0);
    }
  }
}

// ---- tape kernels (forward pieces with a given dt; same per-item code as the step)

template <typename T, int DIM>
__global__ void __launch_bounds__(kFVThreads)
k_tape_stage(FVArgs<T> a, const T* Pin, T* Pout, const T* P0, T h) {
  using G = TileGeom<T, DIM>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const long long ntiles = fv_num_tiles<DIM>(a.n, G::T0, G::T1, G::T2);
  T m[3] = {T(0), T(0), T(0)};
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int o[3];
    tile_origin<DIM>(tile, a.n, G::T0, G::T1, G::T2, o);
    FVItems<T, DIM, RS_HLL, 0>::hydro(a, o, Pin, Pout, P0, h, nullptr, smem, m, false);
  }
}

template <typename T, int DIM>
__global__ void __launch_bounds__(kFVThreads)
k_tape_mag(FVArgs<T> a, const T* Z, T* Zn, T h) {
  const long long nc = a.ncells;
  MagSrc<T, DIM> src = Z ? MagSrc<T, DIM>{Z, Z + 3 * nc, false}
                         : MagSrc<T, DIM>{a.state + (DIM + 2) * nc, a.state + nc, true};
  T change = T(0);
  MagItems<T, DIM>::direct(a, a.state, src, Zn, h, (long long)blockIdx.x * blockDim.x + threadIdx.x, nc,
                           (long long)gridDim.x * blockDim.x, &change);
}

template <typename T, int DIM>
__global__ void __launch_bounds__(kFVThreads)
k_tape_final(FVArgs<T> a, const T* Z, T* out) {
  T m[3] = {T(0), T(0), T(0)};
  MagItems<T, DIM>::finalize(a, a.state, Z, out, (long long)blockIdx.x * blockDim.x + threadIdx.x, a.ncells,
                             (long long)gridDim.x * blockDim.x, false, m);
}

// ------------------------------------------------------------ host side

// One step's slots in the tape: S0 (full state), S1 (gas), S2 (full), the
// iterates Z[0..k] (6 rows each), S3 (full), S4 (gas); S5 is the next
// step's S0.
template <typename T>
struct StepTape {
  T* S0;
  T* S1;
  T* S2;
  T* Z;   // Z[j] = Z + 6 j nc
  T* S3;
  T* S4;
  T* S5;
  int iters;  // k: evaluations after the first
  double dt;
};

// Cotangent buffers of one reverse step.
template <typename T>
struct AdjScratch {
  T* lS4;   // gas rows
  T* lS3;   // full
  T* lS2;   // full
  T* lS1;   // gas
  T* lU;    // gas
  T* lZ0;   // 6 rows
  T* lZ1;
  T* lJ;    // 3
  T* lBa;   // 3
  T* lva;   // 3
  T* lv0;   // 3
};

inline int grid_for(long long nc) {
  const long long b = (nc + kThreads - 1) / kThreads;
  return (int)(b < 4096 ? b : 4096);
}

template <typename T, int DIM, int K, bool FIRST>
int axis_attr() {
  return (int)cudaFuncSetAttribute(k_stage_axis<T, DIM, K, FIRST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)AxisTile<DIM, K>::template smem<T, FIRST>(DIM + 2));
}

template <typename T, int DIM>
int set_attrs() {
  int rc = axis_attr<T, DIM, DIM - 1, true>();
  rc |= axis_attr<T, DIM, 0, false>();
  if (DIM == 3) rc |= axis_attr<T, DIM, 1, false>();
  rc |= (int)cudaFuncSetAttribute(k_tape_stage<T, DIM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)TileGeom<T, DIM>::SMEM);
  return rc ? AMX_ERR_CUDA : AMX_OK;
}

template <typename T, int DIM, int K, bool FIRST>
void launch_axis(const AdjGrid<T>& g, const T* Pin, const T* Pout, const T* P0, const T* lPout, T* lU, T* lPin,
                 T* lP0, int accumulate, T h, cudaStream_t s) {
  using A = AxisTile<DIM, K>;
  const long long blocks = (long long)((g.n + A::L - 1) / A::L) * ((g.n + A::W - 1) / A::W) * (DIM == 3 ? g.n : 1);
  k_stage_axis<T, DIM, K, FIRST><<<(unsigned)blocks, A::THREADS, A::template smem<T, FIRST>(DIM + 2), s>>>(
      g, Pin, Pout, P0, lPout, lU, lPin, lP0, accumulate, h);
}

// Reverse of one hydro stage: lPout -> lPin (set, or added with
// `accumulate`), and the RK2 combination's P0 term into lP0.  The pass along
// the contiguous axis goes first (it forms lU and initialises lPin).
template <typename T, int DIM>
void stage_adjoint(const AdjGrid<T>& g, const T* Pin, const T* Pout, const T* P0, const T* lPout, T* lU, T* lPin,
                   T* lP0, int accumulate, T h, cudaStream_t s) {
  launch_axis<T, DIM, DIM - 1, true>(g, Pin, Pout, P0, lPout, lU, lPin, lP0, accumulate, h, s);
  launch_axis<T, DIM, 0, false>(g, Pin, Pout, P0, lPout, lU, lPin, lP0, accumulate, h, s);
  if (DIM == 3) launch_axis<T, DIM, 1, false>(g, Pin, Pout, P0, lPout, lU, lPin, lP0, accumulate, h, s);
}

// Records one step of the forward (dt, k given) into `t`; S0 is filled.
template <typename T, int DIM>
int tape_step(FVArgs<T> a, const StepTape<T>& t, bool mhd, cudaStream_t s) {
  using G = TileGeom<T, DIM>;
  constexpr int NVG = DIM + 2;
  const long long nc = a.ncells;
  const long long ntiles = fv_num_tiles<DIM>(a.n, G::T0, G::T1, G::T2);
  const unsigned tiles = (unsigned)ntiles;
  const T dtT = T(t.dt);
  const T h = mhd ? dtT / T(2) : dtT;
  k_tape_stage<T, DIM><<<tiles, kFVThreads, G::SMEM, s>>>(a, t.S0, t.S1, nullptr, h);
  T* S2 = mhd ? t.S2 : t.S5;
  // S2 = S0 with the gas rows replaced
  if (mhd && cudaMemcpyAsync(S2 + NVG * nc, t.S0 + NVG * nc, sizeof(T) * 3 * nc, cudaMemcpyDeviceToDevice, s))
    return AMX_ERR_CUDA;
  k_tape_stage<T, DIM><<<tiles, kFVThreads, G::SMEM, s>>>(a, t.S1, S2, t.S0, h);
  if (!mhd) return cudaGetLastError() == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
  FVArgs<T> am = a;
  am.state = S2;
  const int gb = grid_for(nc);
  for (int j = 0; j <= t.iters; ++j)
    k_tape_mag<T, DIM><<<gb, kFVThreads, 0, s>>>(am, j ? t.Z + 6 * (j - 1) * nc : nullptr, t.Z + 6 * j * nc, dtT);
  // the write-back S3 = W(S2, Z_k), out of place (every row of S3 written)
  k_tape_final<T, DIM><<<gb, kFVThreads, 0, s>>>(am, t.Z + 6 * t.iters * nc, t.S3);
  k_tape_stage<T, DIM><<<tiles, kFVThreads, G::SMEM, s>>>(a, t.S3, t.S4, nullptr, h);
  if (cudaMemcpyAsync(t.S5 + NVG * nc, t.S3 + NVG * nc, sizeof(T) * 3 * nc, cudaMemcpyDeviceToDevice, s))
    return AMX_ERR_CUDA;
  k_tape_stage<T, DIM><<<tiles, kFVThreads, G::SMEM, s>>>(a, t.S4, t.S5, t.S3, h);
  return cudaGetLastError() == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
}

// Reverse of one step: lam (cotangent of S5, full state) -> lS0 (full state).
// lam and lS0 may not alias.
template <typename T, int DIM>
int adjoint_step(const AdjGrid<T>& g, const StepTape<T>& t, bool mhd, int midpoint, const T* lam, T* lS0,
                 const AdjScratch<T>& w, cudaStream_t s) {
  constexpr int NVG = DIM + 2;
  const long long nc = g.nc;
  const size_t row = sizeof(T) * (size_t)nc;
  const T dtT = T(t.dt);
  const T h = mhd ? dtT / T(2) : dtT;
  if (!mhd) {
    if (cudaMemsetAsync(lS0, 0, row * NVG, s)) return AMX_ERR_CUDA;
    stage_adjoint<T, DIM>(g, t.S1, t.S5, t.S0, lam, w.lU, w.lS1, lS0, 0, h, s);
    stage_adjoint<T, DIM>(g, t.S0, t.S1, nullptr, w.lS1, w.lU, lS0, nullptr, 1, h, s);
    return cudaGetLastError() == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
  }
  const int gb = grid_for(nc);
  // second half: S5 = C(S3, L(S4)), S4 = L(S3); B rows of S3 pass to S5
  if (cudaMemsetAsync(w.lS3, 0, row * NVG, s)) return AMX_ERR_CUDA;
  if (cudaMemcpyAsync(w.lS3 + NVG * nc, lam + NVG * nc, row * 3, cudaMemcpyDeviceToDevice, s)) return AMX_ERR_CUDA;
  stage_adjoint<T, DIM>(g, t.S4, t.S5, t.S3, lam, w.lU, w.lS4, w.lS3, 0, h, s);
  stage_adjoint<T, DIM>(g, t.S3, t.S4, nullptr, w.lS4, w.lU, w.lS3, nullptr, 1, h, s);
  // write-back and the fixed-point evaluations, last to first
  k_final_adj<T, DIM><<<gb, kThreads, 0, s>>>(g, w.lS3, w.lZ0, w.lS2, w.lv0);
  T* lZn = w.lZ0;
  T* lZp = w.lZ1;
  T* lB0 = w.lS2 + NVG * nc;
  const unsigned mb = mag_adj_blocks<T, DIM>(g.n);
  for (int j = t.iters; j >= 0; --j) {
    const T* Zin = j ? t.Z + 6 * (j - 1) * nc : nullptr;
    k_mag_adj1<T, DIM><<<mb, kThreads, 0, s>>>(g, Zin, t.S2, lZn, dtT, midpoint, w.lJ, w.lBa, w.lva, lB0, w.lv0,
                                               w.lS2);
    k_mag_adj2<T, DIM><<<gb, kThreads, 0, s>>>(g, w.lJ, w.lBa, w.lva, midpoint, j == 0, lZp, lB0, w.lv0, w.lS2);
    T* tmp = lZn; lZn = lZp; lZp = tmp;
  }
  // first half: S2 = C(S0, L(S1)), S1 = L(S0); B rows of S0 pass to S2
  if (cudaMemsetAsync(lS0, 0, row * NVG, s)) return AMX_ERR_CUDA;
  if (cudaMemcpyAsync(lS0 + NVG * nc, lB0, row * 3, cudaMemcpyDeviceToDevice, s)) return AMX_ERR_CUDA;
  stage_adjoint<T, DIM>(g, t.S1, t.S2, t.S0, w.lS2, w.lU, w.lS1, lS0, 0, h, s);
  stage_adjoint<T, DIM>(g, t.S0, t.S1, nullptr, w.lS1, w.lU, lS0, nullptr, 1, h, s);
  return cudaGetLastError() == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
}

}  // namespace adj
}  // namespace amx
