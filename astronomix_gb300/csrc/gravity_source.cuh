// Gravitational source term of the finite-volume scheme (kernels and their
// launcher), shared by the FP32 unit (gravity_f32.cu, fast division) and the
// FP64 one (gravity.cu).
//
// References (astronomix 0.5.1):
//   _physics_modules/_self_gravity/_self_gravity.py:68-337   source term per axis
//   _physics_modules/_self_gravity/_self_gravity.py:341-390  _apply_self_gravity
#pragma once

#include <cuda_runtime.h>

#include "../../include/amx.h"
#include "amx_common.cuh"
#include "fv_kernels.cuh"

namespace amx {

constexpr int kGThreads = 256;
constexpr int kGSeg = 16;  // interfaces per thread of a face sweep

// How the Poisson solve grid maps onto the stored cells.
struct GravGrid {
  int dim;
  int n;     // stored cells per axis
  int goff;  // 2 with ghost-cell handling (the padded grid), 0 otherwise
  int M;     // n + 2 goff: the grid the reference solves on
  int E;     // FFT extent per axis: M (periodic) or 2 M (open, zero padded)
  int roll;  // periodic roll handling: stencil offsets wrap
  AxisBC bc[3];
};

template <typename T>
struct GravSrc {
  const T* old;    // gas rows before the gas update
  T* state;        // gas rows after it (updated in place)
  const T* phi;    // potential on the FFT grid (solve-grid corner)
  T* eacc;         // [ncells] energy source summed over the axes done so far
  GravGrid g;
  long long nc;
  const FVControl* ctl;
  double dt_scale;
  double dx;
  double gamma;
  int version;
  int lm;
  int am;  // AM_HLLC (1) / HYBRID_HLLC (2): the compression switch of the flux; 0 otherwise
  int split;
  int first_order;
  int limiter;
};

__device__ __forceinline__ long long grav_ext_index(const GravGrid& g, const int* p) {
  long long r = p[0];
  for (int k = 1; k < g.dim; ++k) r = r * g.E + p[k];
  return r;
}

// The potential at stored cell ic shifted by o along axis k (solve-grid
// coordinates; wrapped with periodic roll).
template <typename T>
__device__ __forceinline__ T grav_phi(const GravSrc<T>& a, const int* ic, int k, int o) {
  const GravGrid& g = a.g;
  int p[3] = {ic[0] + g.goff, ic[1] + g.goff, ic[2] + g.goff};
  p[k] = g.roll ? wrap(ic[k] + o, g.n) : ic[k] + o + g.goff;
  return a.phi[grav_ext_index(g, p)];
}

// The old state at cell ic with coordinate i along axis k (boundary mapped,
// the axis-normal velocity negated across a reflective wall).
template <typename T, int DIM>
__device__ __forceinline__ void grav_load(const GravSrc<T>& a, const int* ic, int k, int i, T* q) {
  const int n = a.g.n;
  int jc[3] = {ic[0], ic[1], ic[2]};
  bool flip = false;
  jc[k] = a.g.roll ? wrap(i, n) : map_index(i, n, a.g.bc[k], DIM == 1, &flip);
  long long c = jc[0];
  if (DIM >= 2) c = c * n + jc[1];
  if (DIM >= 3) c = c * n + jc[2];
#pragma unroll
  for (int v = 0; v < DIM + 2; ++v) q[v] = a.old[v * a.nc + c];
  if (flip) q[k + 1] = -q[k + 1];
}

// The AM_HLLC / HYBRID_HLLC compression switch (hll.py:268-326, as
// am_compressed forms it) of the old state's cell whose coordinate along
// axis k is j: qm, q0, qp are its cells j - 1, j, j + 1 along k (as grav_load
// maps them); the neighbours along the other axes come from global memory,
// mapped the same way (a reflective wall negates its axis's velocity).
template <typename T, int DIM>
__device__ __forceinline__ bool grav_am_switch(const GravSrc<T>& a, const int* ic, int k, int j, const T* qm,
                                               const T* q0, const T* qp, T gamma, T dxT) {
  const int n = a.g.n;
  bool fk = false;
  int base[3] = {ic[0], ic[1], ic[2]};
  base[k] = a.g.roll ? wrap(j, n) : map_index(j, n, a.g.bc[k], DIM == 1, &fk);
  T div = T(0);
#pragma unroll
  for (int ax = 0; ax < DIM; ++ax) {
    T vp, vm;
    if (ax == k) {
      vp = qp[ax + 1];
      vm = qm[ax + 1];
    } else {
      T v2[2];
#pragma unroll
      for (int sgn = 0; sgn < 2; ++sgn) {
        int jc[3] = {base[0], base[1], base[2]};
        bool f = false;
        const int g = ic[ax] + (sgn ? -1 : 1);
        jc[ax] = a.g.roll ? wrap(g, n) : map_index(g, n, a.g.bc[ax], DIM == 1, &f);
        long long c = jc[0];
        if (DIM >= 2) c = c * n + jc[1];
        if (DIM >= 3) c = c * n + jc[2];
        const T v = a.old[(ax + 1) * a.nc + c];
        v2[sgn] = f ? -v : v;
      }
      vp = v2[0];
      vm = v2[1];
    }
    div = div + (vp - vm) / (T(2) * dxT);
  }
  const T c = sound_speed(q0[0], q0[DIM + 1], gamma);
  return div < T(-0.05) * c / dxT;
}

// The two interface states of the centre cell q0 along axis k (left face
// `lo`, right face `hi`): MUSCL-Hancock (split), limited linear (unsplit),
// or the cell value (first-order fallback) -- _self_gravity.py:125-158.
template <typename T, int DIM>
__device__ __forceinline__ void grav_states(const GravSrc<T>& a, const T* qm, const T* q0, const T* qp, int k, T gamma,
                                            T h, T dxT, T* lo, T* hi) {
  constexpr int NV = DIM + 2;
  if (a.first_order) {
#pragma unroll
    for (int v = 0; v < NV; ++v) lo[v] = hi[v] = q0[v];
  } else if (a.split) {
    muscl_states<T, DIM>(qm, q0, qp, k + 1, gamma, h, dxT, a.limiter, lo, hi);
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const T d = half_slope(qm[v], q0[v], qp[v], a.limiter, dxT);
      lo[v] = q0[v] - d;
      hi[v] = q0[v] + d;
    }
  }
}

// What each cell accounts for of the mass flux through an interface, for
// RIEMANN_SPLIT(_UNSTABLE) (_self_gravity.py:159-284): the HLLC dissipation
// split between the two cells; `to_im1` is the right cell's share, `im1`
// the left cell's.
template <typename T, int DIM>
__device__ __forceinline__ void riemann_split_mass(const T* qL, const T* qR, int d, T gamma, bool lm,
                                                   bool unstable, T* to_im1, T* im1) {
  constexpr int P = DIM + 1;
  const T rhoL = qL[0], uL = qL[d], pL = qL[P];
  const T rhoR = qR[0], uR = qR[d], pR = qR[P];
  const T cL = sound_speed(rhoL, pL, gamma), cR = sound_speed(rhoR, pR, gamma);
  const T FL = uL * rhoL, FR = uR * rhoR;
  const T sL = Num<T>::sqrt_(rhoL), sR = Num<T>::sqrt_(rhoR);
  const T u_hat = (sL * uL + sR * uR) / (sL + sR);
  const T c_hat_sq = (cL * cL * sL + cR * cR * sR) / (sL + sR) +
                     T(0.5) * (sL * sR / ((sL + sR) * (sL + sR))) * ((uR - uL) * (uR - uL));
  const T c_hat = Num<T>::sqrt_(c_hat_sq);
  const T SL = jmin(uL - cL, u_hat - c_hat);
  const T SR = jmax(uR + cR, u_hat + c_hat);
  const T S_star = (pR - pL + rhoL * uL * (SL - uL) - rhoR * uR * (SR - uR)) / (rhoL * (SL - uL) - rhoR * (SR - uR));
  const T USL = rhoL * (SL - uL) / (SL - S_star);
  const T USR = rhoR * (SR - uR) / (SR - S_star);
  T SLs = SL, SRs = SR;
  if (lm) {
    const T Ma = jmax(Num<T>::abs_(uL / cL), Num<T>::abs_(uR / cR));
    const T ph = Num<T>::sin_(jmin(T(1), Ma / T(0.1)) * T(3.141592653589793) / T(2));
    SLs = SL * ph;
    SRs = SR * ph;
  }
  const T diss = T(0.5) * (SLs * (USL - rhoL) + Num<T>::abs_(S_star) * (USL - USR) + SRs * (USR - rhoR));
  T a = T(0.5) * FR + jmin(diss, T(0));
  T b = T(0.5) * FL + jmax(diss, T(0));
  if (unstable) {
    a = (SR <= T(0)) ? FR / T(2) : a;
    a = (SL >= T(0)) ? FL / T(2) : a;
    b = (SL >= T(0)) ? FL / T(2) : b;
    b = (SR <= T(0)) ? FR / T(2) : b;
  }
  *to_im1 = a;
  *im1 = b;
}

// The energy source of axis k for the interface-based versions
// (DONOR_ACCOUNTING, HALF_SPLIT, RIEMANN_SPLIT(_UNSTABLE)): each thread
// walks kGSeg interfaces of one line along k with a sliding window of the
// old state, so that every interface's states and Riemann problem are
// computed once; the cell between two interfaces gets
//   e_k = (its share of the left interface's mass flux) * (-(phi[i] - phi[i-1]) / dx)
//       + (its share of the right one's) * (-(phi[i+1] - phi[i]) / dx)
// and adds it to eacc (axes in order x, y, z, as the reference sums them).
// Threads of a warp take neighbouring lines (the contiguous axis across
// lanes when k is not the last axis).
template <typename T, int DIM, int RS, int K>
__global__ void __launch_bounds__(kGThreads) k_grav_faces(GravSrc<T> a) {
  constexpr int NV = DIM + 2;
  constexpr int k = K;  // the axis: a compile-time index keeps the state windows in registers
  const FVControl* ctl = a.ctl;
  if (!*(volatile const int*)&ctl->active) return;
  const T h = T(*(volatile const double*)&ctl->dt * a.dt_scale);
  const T gamma = T(a.gamma);
  const T dxT = T(a.dx);
  const int n = a.g.n;
  const long long ntrans = a.nc / n;
  const int nseg = (n + kGSeg - 1) / kGSeg;
  const long long total = ntrans * nseg;
  const int version = a.version;
  const bool lm = a.lm != 0;
  const bool rsplit = version == AMX_RIEMANN_SPLIT || version == AMX_RIEMANN_SPLIT_UNSTABLE;
  const bool unstable = version == AMX_RIEMANN_SPLIT_UNSTABLE;
  const T alpha = T(((volatile const double*)ctl->seam_maxima)[k]);
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < total;
       w += (long long)gridDim.x * blockDim.x) {
    const long long t = w % ntrans;
    const int seg = (int)(w / ntrans);
    int ic[3] = {0, 0, 0};
    {
      long long r = t;
      for (int d = DIM - 1; d >= 0; --d) {
        if (d == k) continue;
        ic[d] = (int)(r % n);
        r /= n;
      }
    }
    const int i0 = seg * kGSeg;
    const int i1 = min(i0 + kGSeg, n);
    // window: w0..w3 = cells j-2 .. j+1 around interface j-1/2
    T w0[NV], w1[NV], w2[NV], w3[NV], lo[NV], hi[NV], hiL[NV];
    grav_load<T, DIM>(a, ic, k, i0 - 2, w0);
    grav_load<T, DIM>(a, ic, k, i0 - 1, w1);
    grav_load<T, DIM>(a, ic, k, i0, w2);
    grav_states<T, DIM>(a, w0, w1, w2, k, gamma, h, dxT, lo, hiL);  // the right state of cell i0 - 1
    T pm2 = grav_phi(a, ic, k, i0 - 2), pm1 = grav_phi(a, ic, k, i0 - 1);
    T share_right = T(0);  // the to_im1 share of cell j - 1 (from interface j - 3/2)
    int jc[3] = {ic[0], ic[1], ic[2]};
    for (int j = i0; j <= i1; ++j) {
      grav_load<T, DIM>(a, ic, k, j + 1, w3);
      grav_states<T, DIM>(a, w1, w2, w3, k, gamma, h, dxT, lo, hi);  // states of cell j
      T to_im1, im1;
      if (rsplit) {
        riemann_split_mass<T, DIM>(hiL, lo, k + 1, gamma, lm, unstable, &to_im1, &im1);
      } else {
        T F[NV];
        bool lmf = lm;
        if constexpr (RS == RS_AM) lmf = grav_am_switch<T, DIM>(a, ic, k, j, w1, w2, w3, gamma, dxT);
        riemann<T, DIM, RS>(hiL, lo, k + 1, gamma, alpha, lmf, F, a.am == 1);
        if (version == AMX_DONOR_ACCOUNTING) {
          to_im1 = jmin(F[0], T(0));
          im1 = jmax(F[0], T(0));
        } else {  // HALF_SPLIT
          to_im1 = T(0.5) * F[0];
          im1 = T(0.5) * F[0];
        }
      }
      const T p0 = grav_phi(a, ic, k, j);
      if (j > i0) {
        // cell j - 1 has both interfaces now
        const T acc_b = -(pm1 - pm2) / dxT;
        const T acc_f = -(p0 - pm1) / dxT;
        const T e = share_right * acc_b + im1 * acc_f;
        jc[k] = j - 1;
        long long c = jc[0];
        if (DIM >= 2) c = c * n + jc[1];
        if (DIM >= 3) c = c * n + jc[2];
        a.eacc[c] = (k == 0) ? e : a.eacc[c] + e;
      }
      share_right = to_im1;
      pm2 = pm1;
      pm1 = p0;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        hiL[v] = hi[v];
        w1[v] = w2[v];
        w2[v] = w3[v];
      }
    }
  }
}

// k_grav_faces for the contiguous (last) axis: the lanes of a warp take 32
// neighbouring cells of one line (coalesced loads), each the states of its
// own cell; the interface left of a lane's cell takes the left neighbour's
// right state by a shuffle, and a cell's right interface share comes from the
// next lane.  A warp completes the 30 cells of lanes 1 .. 30.
template <typename T, int DIM, int RS>
__global__ void __launch_bounds__(kGThreads) k_grav_faces_last(GravSrc<T> a) {
  constexpr int NV = DIM + 2;
  constexpr int k = DIM - 1;
  constexpr int kCells = 30;
  const FVControl* ctl = a.ctl;
  if (!*(volatile const int*)&ctl->active) return;
  const T h = T(*(volatile const double*)&ctl->dt * a.dt_scale);
  const T gamma = T(a.gamma);
  const T dxT = T(a.dx);
  const int n = a.g.n;
  const long long ntrans = a.nc / n;
  const int nseg = (n + kCells - 1) / kCells;
  const long long total = ntrans * nseg;  // warps
  const int version = a.version;
  const bool lm = a.lm != 0;
  const bool rsplit = version == AMX_RIEMANN_SPLIT || version == AMX_RIEMANN_SPLIT_UNSTABLE;
  const bool unstable = version == AMX_RIEMANN_SPLIT_UNSTABLE;
  const T alpha = T(((volatile const double*)ctl->seam_maxima)[k]);
  const int lane = threadIdx.x & 31;
  const long long warps_per_grid = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long w = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < total; w += warps_per_grid) {
    const long long t = w % ntrans;
    const int seg = (int)(w / ntrans);
    int ic[3] = {0, 0, 0};
    {
      long long r = t;
      for (int d = DIM - 2; d >= 0; --d) {
        ic[d] = (int)(r % n);
        r /= n;
      }
    }
    // this lane's cell (clamped into the mapped range; lanes past the line end compute unused values)
    const int jr = seg * kCells - 1 + lane;
    const int j = jr < n ? jr : n;
    T qm[NV], q0[NV], qp[NV], lo[NV], hi[NV];
    grav_load<T, DIM>(a, ic, k, j - 1, qm);
    grav_load<T, DIM>(a, ic, k, j, q0);
    grav_load<T, DIM>(a, ic, k, j + 1, qp);
    grav_states<T, DIM>(a, qm, q0, qp, k, gamma, h, dxT, lo, hi);
    // interface j - 1/2: the left cell's right state from the previous lane
    T hiL[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) hiL[v] = __shfl_up_sync(0xffffffffu, hi[v], 1);
    T to_im1 = T(0), im1 = T(0);
    if (lane > 0) {
      if (rsplit) {
        riemann_split_mass<T, DIM>(hiL, lo, k + 1, gamma, lm, unstable, &to_im1, &im1);
      } else {
        T F[NV];
        bool lmf = lm;
        if constexpr (RS == RS_AM) lmf = grav_am_switch<T, DIM>(a, ic, k, j, qm, q0, qp, gamma, dxT);
        riemann<T, DIM, RS>(hiL, lo, k + 1, gamma, alpha, lmf, F, a.am == 1);
        if (version == AMX_DONOR_ACCOUNTING) {
          to_im1 = jmin(F[0], T(0));
          im1 = jmax(F[0], T(0));
        } else {  // HALF_SPLIT
          to_im1 = T(0.5) * F[0];
          im1 = T(0.5) * F[0];
        }
      }
    }
    // the share of this cell's right interface, computed by the next lane
    const T share_r = __shfl_down_sync(0xffffffffu, im1, 1);
    if (lane >= 1 && lane <= kCells && jr < n) {
      const T pm = grav_phi(a, ic, k, jr - 1), p0 = grav_phi(a, ic, k, jr), pp = grav_phi(a, ic, k, jr + 1);
      const T acc_b = -(p0 - pm) / dxT;
      const T acc_f = -(pp - p0) / dxT;
      const T e = to_im1 * acc_b + share_r * acc_f;
      int jc[3] = {ic[0], ic[1], ic[2]};
      jc[k] = jr;
      long long c = jc[0];
      if (DIM >= 2) c = c * n + jc[1];
      if (DIM >= 3) c = c * n + jc[2];
      a.eacc[c] = (k == 0) ? e : a.eacc[c] + e;
    }
  }
}

// The update of _apply_self_gravity (_self_gravity.py:341-390), one cell per
// thread: momentum source rho a_k with the central acceleration
// a_k = -(phi[i+1] - phi[i-1]) / 2dx, energy source rho v_k a_k summed over
// the axes (SIMPLE_SOURCE_TERM) or the interface sum in eacc, then
// U += dt S in conserved variables and back to primitives.
template <typename T, int DIM>
__global__ void __launch_bounds__(kGThreads) k_grav_update(GravSrc<T> a) {
  constexpr int NV = DIM + 2, P = DIM + 1;
  const FVControl* ctl = a.ctl;
  if (!*(volatile const int*)&ctl->active) return;
  const T h = T(*(volatile const double*)&ctl->dt * a.dt_scale);
  const T gamma = T(a.gamma);
  const T two_dx = T(2.0 * a.dx);
  const int n = a.g.n;
  const long long nc = a.nc;
  const bool simple = a.version == AMX_SIMPLE_SOURCE_TERM;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
    int ic[3] = {0, 0, 0};
    {
      long long r = c;
      for (int k = DIM - 1; k >= 0; --k) {
        ic[k] = (int)(r % n);
        r /= n;
      }
    }
    const T rho = a.old[c];
    T mS[DIM];
    T eS = T(0);
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const T acc = -(grav_phi(a, ic, k, 1) - grav_phi(a, ic, k, -1)) / two_dx;
      mS[k] = rho * acc;
      if (simple) {
        const T e = rho * a.old[(k + 1) * nc + c] * acc;
        eS = (k == 0) ? e : eS + e;
      }
    }
    if (!simple) eS = a.eacc[c];
    T qn[NV], U[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) qn[v] = a.state[v * nc + c];
    prim_to_cons<T, DIM>(qn, U, gamma);
#pragma unroll
    for (int k = 0; k < DIM; ++k) U[k + 1] = U[k + 1] + h * mS[k];
    U[P] = U[P] + h * eS;
    cons_to_prim<T, DIM>(U, qn, gamma);
#pragma unroll
    for (int v = 0; v < NV; ++v) a.state[v * nc + c] = qn[v];
  }
}

inline int grav_grid_for(long long work, int num_sms) {
  const long long b = (work + kGThreads - 1) / kGThreads;
  const long long cap = (long long)num_sms * 8;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

template <typename T, int DIM, int K>
void grav_faces_axis(const GravSrc<T>& a, int rs, int num_sms, cudaStream_t s) {
  const long long ntrans = a.nc / a.g.n;
  if (K == DIM - 1) {
    // one warp per 30 cells of a line along the contiguous axis
    const long long warps = ntrans * ((a.g.n + 29) / 30);
    const int grid = grav_grid_for(warps * 32, num_sms);
    if (rs == AMX_LAX_FRIEDRICHS) k_grav_faces_last<T, DIM, RS_LF><<<grid, kGThreads, 0, s>>>(a);
    else if (rs == AMX_HLL) k_grav_faces_last<T, DIM, RS_HLL><<<grid, kGThreads, 0, s>>>(a);
    else if (a.am) k_grav_faces_last<T, DIM, RS_AM><<<grid, kGThreads, 0, s>>>(a);
    else k_grav_faces_last<T, DIM, RS_HLLC><<<grid, kGThreads, 0, s>>>(a);
    return;
  }
  const int grid = grav_grid_for(ntrans * ((a.g.n + kGSeg - 1) / kGSeg), num_sms);
  if (rs == AMX_LAX_FRIEDRICHS) k_grav_faces<T, DIM, RS_LF, K><<<grid, kGThreads, 0, s>>>(a);
  else if (rs == AMX_HLL) k_grav_faces<T, DIM, RS_HLL, K><<<grid, kGThreads, 0, s>>>(a);
  else if (a.am) k_grav_faces<T, DIM, RS_AM, K><<<grid, kGThreads, 0, s>>>(a);
  else k_grav_faces<T, DIM, RS_HLLC, K><<<grid, kGThreads, 0, s>>>(a);
}

template <typename T, int DIM>
int grav_source_dim(const GravSrc<T>& a, int rs, int num_sms, cudaStream_t s) {
  if (a.version != AMX_SIMPLE_SOURCE_TERM) {
    grav_faces_axis<T, DIM, 0>(a, rs, num_sms, s);
    if (DIM >= 2) grav_faces_axis<T, DIM, (DIM >= 2 ? 1 : 0)>(a, rs, num_sms, s);
    if (DIM >= 3) grav_faces_axis<T, DIM, (DIM >= 3 ? 2 : 0)>(a, rs, num_sms, s);
  }
  k_grav_update<T, DIM><<<grav_grid_for(a.nc, num_sms), kGThreads, 0, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
}

// The source term and update of one gas update (the launches of every axis).
template <typename T>
int grav_source_launch(const GravSrc<T>& a, int rs, int num_sms, cudaStream_t s) {
  switch (a.g.dim) {
    case 1: return grav_source_dim<T, 1>(a, rs, num_sms, s);
    case 2: return grav_source_dim<T, 2>(a, rs, num_sms, s);
    default: return grav_source_dim<T, 3>(a, rs, num_sms, s);
  }
}

}  // namespace amx
