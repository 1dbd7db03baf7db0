// Finite-difference WENO-CT MHD step: kernels and their typed launchers.
//
// One time step = 1 CFL reduction + 5 SSPRK(5,4) stages x 7 sweeps + 1
// finalize sweep, all stream-ordered launches that read dt from the device
// control block (no host round trip per step).  Stage s:
//
//   prep      q <- positivity(q); qc <- update_cell_center_fields(q, b)
//   weno x/y/z   interface fluxes of qc; acc += F[i+1/2] - F[i-1/2];
//             CT flux corrections F_d[B_t] + c2f(B_d) c2f(v_t) at the faces
//   emf       edge EMFs Omega from the corrected fluxes (4th-order c2f)
//   emf_avg   point values -> averages
//   update    rhs = -dt/dx acc, rb = curl_6(Omega); RK combination of q, b
//             and accumulation into q_final, b_final
//
// and finalize: q_final <- ucc(q_final, b_final), positivity, primitives.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

#include "fd_api.h"
#include "fd_kernels.cuh"

namespace amx {
namespace fd {

// SSPRK(5,4) coefficients (_ssprk.py:247-272)
static __constant__ double kRHS[5] = {0.39175222700392, 0.36841059262959, 0.25189177424738, 0.54497475021237,
                               0.22600748319395};
static __constant__ double kK0[5] = {1.0, 0.44437049406734, 0.62010185138540, 0.17807995410773, -2.081261929715610e-02};
static __constant__ double kKC[5] = {0.0, 0.55562950593266, 0.37989814861460, 0.82192004589227, 5.03580947213895e-01};
static __constant__ double kFIN[5] = {-2.081261929715610e-02, 0.0, 0.51723167208978, -6.518979800418380e-12,
                               5.03580947213895e-01};

constexpr int kThreads = 256;

template <typename T>
struct Bufs {
  T* P;    // state (prim, 11 rows)
  T* Q0;   // 8
  T* Q;    // 8
  T* QF;   // 8
  T* QC;   // 8
  T* ACC;  // 8
  T* B;    // 3  current face fields
  T* BF;   // 3  final accumulator of the faces
  T* M;    // 6  CT-corrected face fluxes: By_fx Bz_fx Bx_fy Bz_fy Bx_fz By_fz
  T* OM;   // 3  edge EMFs Omega_x, Omega_y, Omega_z (point values)
  T* OB;   // 3  edge EMFs (averages)
  FDControl* ctl;
  T* WS;   // stellar wind: [5][wind_n^3] source of the current stage
  FDArgs a;
};

#define FD_ACTIVE_OR_RETURN(ctl) \
  if (!*(volatile int*)&(ctl)->active) return;

// ---------------------------------------------------------------- CFL

template <typename T>
__global__ void __launch_bounds__(kThreads) k_cfl(Bufs<T> b) {
  __shared__ double red[32];
  const FDArgs a = b.a;
  const T gamma = T(a.gamma), rhomin = T(a.rhomin), pgmin = T(a.pgmin);
  const long long nc = a.nc;
  T m[3] = {T(0), T(0), T(0)};
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
    T P[8], U[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) P[r] = b.P[r * nc + c];
    prim_to_cons(P, U, gamma);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      T Up[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) Up[r] = U[perm_row(d, r)];
      T vx, cf, ca, cs;
      eigenvalue_blocks(Up, gamma, rhomin, pgmin, &vx, &cf, &ca, &cs);
      T l = Num<T>::abs_(vx - cf);
      l = nanmax(l, Num<T>::abs_(vx - ca));
      l = nanmax(l, Num<T>::abs_(vx - cs));
      l = nanmax(l, Num<T>::abs_(vx));
      l = nanmax(l, Num<T>::abs_(vx + cs));
      l = nanmax(l, Num<T>::abs_(vx + ca));
      l = nanmax(l, Num<T>::abs_(vx + cf));
      m[d] = nanmax(m[d], l);
    }
  }
  for (int d = 0; d < 3; ++d) {
    const double r = block_max<double>((double)m[d], red);
    if (threadIdx.x == 0) atomic_max_nonneg(&b.ctl->lam[d], r);
  }
  // the last block to finish turns the maxima into dt
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(&b.ctl->done_count, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    FDControl* ctl = b.ctl;
    volatile unsigned long long* lam = ctl->lam;
    const double lx = bits_to_double(lam[0]), ly = bits_to_double(lam[1]), lz = bits_to_double(lam[2]);
    const double t = ctl->t;
    double dt;
    int active;
    if (a.fixed_timestep) {
      dt = a.dt_fixed;
      active = 1;
    } else {
      dt = a.C_cfl * a.dx / (lx + ly + lz);
      dt = fmin(dt, a.dt_max);
      active = (t < a.t_end) ? 1 : 0;
    }
    if (!(t < a.t_pause)) active = 0;
    if (a.exact_end_time) dt = fmin(dt, a.t_end - t);
    if (dt != dt) raise_status(&ctl->status, AMX_ERR_NAN);
    ctl->dt = dt;
    ctl->active = active;
    lam[0] = 0ull;
    lam[1] = 0ull;
    lam[2] = 0ull;
    ctl->done_count = 0u;
    __threadfence();
  }
}

// ---------------------------------------------------------------- cell-centre B refresh

// update_cell_center_fields (_constrained_transport.py:161-198) for one cell
template <typename T>
__device__ __forceinline__ void ucc(T* U, const T* bx, const T* by, const T* bz, int i, int j, int k, int n) {
  const T b2_old = U[BX] * U[BX] + U[BY] * U[BY] + U[BZ] * U[BZ];
  U[BX] = f2c(bx[nb(i, j, k, 0, -3, n)], bx[nb(i, j, k, 0, -2, n)], bx[nb(i, j, k, 0, -1, n)], bx[cidx(i, j, k, n)],
              bx[nb(i, j, k, 0, 1, n)], bx[nb(i, j, k, 0, 2, n)]);
  U[BY] = f2c(by[nb(i, j, k, 1, -3, n)], by[nb(i, j, k, 1, -2, n)], by[nb(i, j, k, 1, -1, n)], by[cidx(i, j, k, n)],
              by[nb(i, j, k, 1, 1, n)], by[nb(i, j, k, 1, 2, n)]);
  U[BZ] = f2c(bz[nb(i, j, k, 2, -3, n)], bz[nb(i, j, k, 2, -2, n)], bz[nb(i, j, k, 2, -1, n)], bz[cidx(i, j, k, n)],
              bz[nb(i, j, k, 2, 1, n)], bz[nb(i, j, k, 2, 2, n)]);
  const T b2_new = U[BX] * U[BX] + U[BY] * U[BY] + U[BZ] * U[BZ];
  U[EN] = U[EN] + T(0.5) * (b2_new - b2_old);
}

// stage prep: positivity of q (stages 0-3) and the cell-centre refresh qc.
// Stage 0 also forms q0 = cons(P) and the initial final-accumulators.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_prep(Bufs<T> b, int stage) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const FDArgs a = b.a;
  const T gamma = T(a.gamma), rhomin = T(a.rhomin), pgmin = T(a.pgmin);
  const long long nc = a.nc;
  const int n = a.n;
  const T* faces = (stage == 0) ? b.P + 8 * nc : b.B;
  const T f0 = T(kFIN[0]);
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
    T U[8];
    if (stage == 0) {
      T P[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) P[r] = b.P[r * nc + c];
      prim_to_cons(P, U, gamma);
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        b.Q0[r * nc + c] = U[r];
        b.QF[r * nc + c] = f0 * U[r];
      }
#pragma unroll
      for (int r = 0; r < 3; ++r) b.BF[r * nc + c] = f0 * faces[r * nc + c];
    } else {
#pragma unroll
      for (int r = 0; r < 8; ++r) U[r] = b.Q[r * nc + c];
    }
    if (stage < 4 && a.enforce_positivity) positivity(U, gamma, rhomin, pgmin);
    if (stage == 0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) b.Q[r * nc + c] = U[r];
    } else if (stage < 4 && a.enforce_positivity) {
      b.Q[RHO * nc + c] = U[RHO];
      b.Q[EN * nc + c] = U[EN];
    }
    int i, j, k;
    decompose(c, n, &i, &j, &k);
    ucc(U, faces, faces + nc, faces + 2 * nc, i, j, k, n);
#pragma unroll
    for (int r = 0; r < 8; ++r) b.QC[r * nc + c] = U[r];
  }
}

// ---------------------------------------------------------------- WENO

// Line tiles of A cells along the flux axis x 32 lanes across it; every
// staged cell (A + 6 with the halo of 3) costs a flux and an eigensystem, so
// longer tiles recompute less halo.  One block per SM leaves the shared
// memory free: FP32 47 cells (212 KB; the 48 x 32 interfaces are six tasks
// per thread; 256^3 step 0.097 s with 7 cells, 0.087 with 15, 0.084 with 31,
// 0.082 with 47), FP64 15 cells (what fits in 227 KB).
template <typename T> struct WenoTile {
  static constexpr int A = sizeof(T) == 4 ? 47 : 15;  // cells per tile along the flux axis
  static constexpr int L = 32;                        // lanes per tile across it
  static constexpr int AH = A + 6;                    // staged cells along the axis (halo 3)
};
constexpr int kCellVals = 24;     // U(8) F(8) rho' vx vy vz h (5) cf ca cs (3)

template <typename T>
constexpr size_t weno_smem() {
  return sizeof(T) * ((size_t)WenoTile<T>::AH * WenoTile<T>::L * kCellVals +
                      (size_t)(WenoTile<T>::A + 1) * WenoTile<T>::L * 8);
}

__device__ __forceinline__ int pmod(int g, int n) {
  int r = g % n;
  return r < 0 ? r + n : r;
}

// Interface fluxes along axis D (0 = x, 1 = y, 2 = z), _weno.py:112-324.
// One block per SM: the characteristic projection needs about 250 registers
// per thread; held to 128 (two blocks) it spilled 440 bytes per thread and
// ran 18 % slower on the 256^3 blast.
template <typename T, int D>
__global__ void __launch_bounds__(kThreads, 1) k_weno(Bufs<T> b) {
  constexpr int kA = WenoTile<T>::A, kL = WenoTile<T>::L, kAH = WenoTile<T>::AH;
  FD_ACTIVE_OR_RETURN(b.ctl);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* S = reinterpret_cast<T*>(smem_raw);          // [kAH][kL][kCellVals]
  T* FI = S + (size_t)kAH * kL * kCellVals;      // [kA+1][kL][8] (permuted frame)
  const FDArgs a = b.a;
  const T gamma = T(a.gamma), rhomin = T(a.rhomin), pgmin = T(a.pgmin);
  const bool floors = a.enforce_positivity != 0;
  const int n = a.n;
  const long long nc = a.nc;
  // tile: along-axis start a0, lane start l0, third coordinate t3
  const int a0 = blockIdx.x * kA;
  const int l0 = blockIdx.y * kL;
  const int t3 = blockIdx.z;

  auto cell_of = [&](int ga, int gl) -> long long {
    // D = 0: along x, lanes z, third y;  D = 1: along y, lanes z, third x;
    // D = 2: along z, lanes y, third x
    if (D == 0) return cidx(ga, t3, gl, n);
    if (D == 1) return cidx(t3, ga, gl, n);
    return cidx(t3, gl, ga, n);
  };

  // ---- stage the cells a0-3 .. a0+kA+2 (permuted frame)
  for (int e = threadIdx.x; e < kAH * kL; e += blockDim.x) {
    int ai, li;
    if (D == 2) { ai = e % kAH; li = e / kAH; }
    else { li = e % kL; ai = e / kL; }
    const int ga = pmod(a0 - 3 + ai, n);
    int gl = l0 + li;
    if (gl >= n) gl = n - 1;
    const long long c = cell_of(ga, gl);
    T* s = S + ((size_t)ai * kL + li) * kCellVals;
    T U[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) U[r] = b.QC[perm_row(D, r) * nc + c];
    T F[8], ev[5];
    mhd_flux(U, F, gamma, rhomin, pgmin, floors);
    eigvec_cell(U, gamma, rhomin, pgmin, ev);
    T vx, cf, ca, cs;
    eigenvalue_blocks(U, gamma, rhomin, pgmin, &vx, &cf, &ca, &cs);
#pragma unroll
    for (int r = 0; r < 8; ++r) { s[r] = U[r]; s[8 + r] = F[r]; }
#pragma unroll
    for (int r = 0; r < 5; ++r) s[16 + r] = ev[r];
    s[21] = cf;
    s[22] = ca;
    s[23] = cs;
  }
  __syncthreads();

  // ---- interfaces a0-1 .. a0+kA-1 (local ii = 0..kA): cell i = a0-1+ii is smem row ii+2
  for (int task = threadIdx.x; task < (kA + 1) * kL; task += blockDim.x) {
    const int li = task % kL, ii = task / kL;
    const T* cst[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) cst[m] = S + ((size_t)(ii + m) * kL + li) * kCellVals;
    // eigenvector blocks from cells i (stencil 2) and i+1 (stencil 3)
    EigIF<T> e;
    eig_interface(cst[2] + 16, cst[3] + 16, cst[2][BX], cst[2][BY], cst[2][BZ], cst[3][BX], cst[3][BY], cst[3][BZ],
                  gamma, e);
    T Fint[8];
#pragma unroll
    for (int r = 0; r < 8; ++r)
      Fint[r] = T(1.0 / 12.0) * (-cst[1][8 + r] + T(7) * cst[2][8 + r] + T(7) * cst[3][8 + r] - cst[4][8 + r]);
#pragma unroll 1
    for (int s = 0; s < 7; ++s) {
      T L[8];
      L_row(e, s, L);
      T sv[6], qv[6];
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        T as = L[0] * cst[m][8], aq = L[0] * cst[m][0];
#pragma unroll
        for (int r = 1; r < 8; ++r) {
          as = as + L[r] * cst[m][8 + r];
          aq = aq + L[r] * cst[m][r];
        }
        sv[m] = as;
        qv[m] = aq;
      }
      T d[5], dq[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) { d[k] = sv[k + 1] - sv[k]; dq[k] = qv[k + 1] - qv[k]; }
      // alpha_s: max |lambda_s| over the six stencil cells (cell centred)
      T amx = T(0);
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        const T vx = cst[m][17], cf = cst[m][21], ca = cst[m][22], cs = cst[m][23];
        T lam;
        switch (s) {
          case 0: lam = vx - cf; break;
          case 1: lam = vx - ca; break;
          case 2: lam = vx - cs; break;
          case 3: lam = vx; break;
          case 4: lam = vx + cs; break;
          case 5: lam = vx + ca; break;
          default: lam = vx + cf; break;
        }
        amx = (m == 0) ? Num<T>::abs_(lam) : jmax(amx, Num<T>::abs_(lam));
      }
      const T second = weno_phi(T(0.5) * (d[0] + amx * dq[0]), T(0.5) * (d[1] + amx * dq[1]),
                                T(0.5) * (d[2] + amx * dq[2]), T(0.5) * (d[3] + amx * dq[3]));
      const T third = weno_phi(T(0.5) * (d[4] - amx * dq[4]), T(0.5) * (d[3] - amx * dq[3]),
                               T(0.5) * (d[2] - amx * dq[2]), T(0.5) * (d[1] - amx * dq[1]));
      const T Fs = -second + third;
      T R[8];
      R_col(e, s, R);
#pragma unroll
      for (int r = 0; r < 8; ++r) Fint[r] = Fint[r] + R[r] * Fs;
    }
    T* fo = FI + ((size_t)ii * kL + li) * 8;
#pragma unroll
    for (int r = 0; r < 8; ++r) fo[r] = Fint[r];
  }
  __syncthreads();

  // ---- cells a0 .. a0+kA-1: flux difference into acc, CT-corrected fluxes at their faces
  // lab rows of the two tangential B components whose fluxes CT corrects
  constexpr int T1 = (D == 0) ? BY : BX;
  constexpr int T2 = (D == 2) ? BY : BZ;
  for (int task = threadIdx.x; task < kA * kL; task += blockDim.x) {
    int ci, li;
    if (D == 2) { ci = task % kA; li = task / kA; }
    else { li = task % kL; ci = task / kL; }
    const int ga = a0 + ci, gl = l0 + li;
    if (ga >= n || gl >= n) continue;
    const long long c = cell_of(ga, gl);
    const T* fr = FI + ((size_t)(ci + 1) * kL + li) * 8;  // face i+1/2
    const T* fl = FI + ((size_t)ci * kL + li) * 8;        // face i-1/2
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int pr = perm_row(D, r);
      const T dF = fr[pr] - fl[pr];
      if (D == 0) b.ACC[r * nc + c] = dF;
      else b.ACC[r * nc + c] = b.ACC[r * nc + c] + dF;
    }
    // c2f over cells i-1 .. i+2 (smem rows ci+2 .. ci+5) of B_d and v_t (lab frame)
    const T* sm = S + ((size_t)(ci + 2) * kL + li) * kCellVals;  // cell i-1
    const T* s0 = sm + kL * kCellVals;                           // cell i
    const T* s1 = s0 + kL * kCellVals;
    const T* s2 = s1 + kL * kCellVals;
    const T Bn = c2f(sm[BX], s0[BX], s1[BX], s2[BX]);  // permuted-frame x = lab axis D
    const int m1 = perm_row(D, T1 - BX + MX), m2 = perm_row(D, T2 - BX + MX);
    const T v1 = c2f(sm[m1] / sm[RHO], s0[m1] / s0[RHO], s1[m1] / s1[RHO], s2[m1] / s2[RHO]);
    const T v2 = c2f(sm[m2] / sm[RHO], s0[m2] / s0[RHO], s1[m2] / s1[RHO], s2[m2] / s2[RHO]);
    b.M[(2 * D) * nc + c] = fr[perm_row(D, T1)] + Bn * v1;
    b.M[(2 * D + 1) * nc + c] = fr[perm_row(D, T2)] + Bn * v2;
  }
}

// ---------------------------------------------------------------- CT

// edge EMFs (_constrained_transport.py:104-131)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_emf(Bufs<T> b) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const int n = b.a.n;
  const long long nc = b.a.nc;
  const T* By_fx = b.M;
  const T* Bz_fx = b.M + nc;
  const T* Bx_fy = b.M + 2 * nc;
  const T* Bz_fy = b.M + 3 * nc;
  const T* Bx_fz = b.M + 4 * nc;
  const T* By_fz = b.M + 5 * nc;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(c, n, &i, &j, &k);
    auto I = [&](const T* f, int ax) {
      return c2f(f[nb(i, j, k, ax, -1, n)], f[c], f[nb(i, j, k, ax, 1, n)], f[nb(i, j, k, ax, 2, n)]);
    };
    const T Oz = I(Bx_fy, 0) - I(By_fx, 1);
    const T Ox = I(By_fz, 1) - I(Bz_fy, 2);
    const T Oy = I(Bz_fx, 2) - I(Bx_fz, 0);
    b.OM[c] = Ox;
    b.OM[nc + c] = Oy;
    b.OM[2 * nc + c] = Oz;
  }
}

// point values -> averages (_interpolate.py:39-62)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_emf_avg(Bufs<T> b) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const int n = b.a.n;
  const long long nc = b.a.nc;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(c, n, &i, &j, &k);
    auto avg = [&](const T* q, int A, int B) {
      const T q0 = q[c];
      const T sx = (q[nb(i, j, k, A, -1, n)] - T(2) * q0 + q[nb(i, j, k, A, 1, n)]) / T(24);
      const T sy = (q[nb(i, j, k, B, -1, n)] - T(2) * q0 + q[nb(i, j, k, B, 1, n)]) / T(24);
      return q0 + sx + sy;
    };
    b.OB[c] = avg(b.OM, 1, 2);                 // Omega_x: (y, z)
    b.OB[nc + c] = avg(b.OM + nc, 0, 2);       // Omega_y: (x, z)
    b.OB[2 * nc + c] = avg(b.OM + 2 * nc, 0, 1);  // Omega_z: (x, y)
  }
}

// The stellar-wind EI source of one cell over the stage's k2 dt
// (stellar_wind.py:485-584), added to the stage's right-hand side
// (_ssprk.py:230-241): the tapered mask (1 inside r_inj, linear to 0 at
// 1.3 r_inj), mass drho/dt = Mdot / V, thermal energy 1/2 v_inf^2 Mdot / V,
// and the momentum rescaled by sqrt(1 + drho / rho) - 1 so the kinetic
// energy stays.  q: the stage's cell-centre-refreshed conserved state.
// Returns false (no source) outside the taper.
template <typename T>
__device__ __forceinline__ bool wind_source(const FDArgs& a, int i, int j, int k, const T* qc, long long nc,
                                            long long c, T dtw, T* src) {
  const double dx = a.dx, half = a.box / 2;
  // helper_data.r: cell centres dx/2 + i dx, distance from the box centre
  const double x = dx / 2 + i * dx - half, y = dx / 2 + j * dx - half, z = dx / 2 + k * dx - half;
  const double r = sqrt(x * x + y * y + z * z);
  if (!(r <= a.wind_r1)) return false;
  const double mask = (r <= a.wind_rinj) ? 1.0 : (a.wind_r1 - r) / (a.wind_r1 - a.wind_rinj);
  const double drho_dt = a.wind_mdot / a.wind_V;
  const double dtd = (double)dtw;
  src[0] = T(drho_dt * mask * dtd);
  const double dE = 0.5 * (a.wind_vinf * a.wind_vinf) * a.wind_mdot / a.wind_V * dtd;
  const double f = sqrt(1.0 + drho_dt * dtd * mask / (double)qc[c]) - 1.0;
#pragma unroll
  for (int r_ = 1; r_ <= 3; ++r_) src[r_] = T((double)qc[r_ * nc + c] * f);
  src[4] = T(dE * mask);
  return true;
}

// The wind source of one stage over the cube of cells that holds the taper
// (zero outside it), before k_update adds it to the right-hand side.  Its
// own kernel, so that the FP64 arithmetic does not weigh on the update's
// registers.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_wind_source(Bufs<T> b, int stage) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const FDArgs a = b.a;
  const int n = a.n, wn = a.wind_n, lo = a.wind_lo;
  const long long nc = a.nc, wn3 = (long long)wn * wn * wn;
  const T dt = T(*(volatile double*)&b.ctl->dt);
  const T k2 = T(kRHS[stage]);
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < wn3; w += (long long)gridDim.x * blockDim.x) {
    const int wi = (int)(w / ((long long)wn * wn)), wj = (int)((w / wn) % wn), wk = (int)(w % wn);
    const int i = lo + wi, j = lo + wj, k = lo + wk;
    const long long c = cidx(i, j, k, n);
    T src[5] = {T(0), T(0), T(0), T(0), T(0)};
    wind_source<T>(a, i, j, k, b.QC, nc, c, k2 * dt, src);
#pragma unroll
    for (int r = 0; r < 5; ++r) b.WS[r * wn3 + w] = src[r];
  }
}

// RHS and the SSPRK(5,4) combination (_ssprk.py:224-228, :298-310, :328-332)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_update(Bufs<T> b, int stage) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const FDArgs a = b.a;
  const int n = a.n;
  const long long nc = a.nc;
  const T dt = T(*(volatile double*)&b.ctl->dt);
  const T k2 = T(kRHS[stage]);
  const T dtdx = k2 * dt / T(a.dx);
  const T k0 = T(kK0[stage]), kc = T(kKC[stage]);
  const T f = (stage < 4) ? T(kFIN[stage + 1]) : T(0);
  const T* bcur = (stage == 0) ? b.P + 8 * nc : b.B;
  const T* b0 = b.P + 8 * nc;
  const T* Ox = b.OB;
  const T* Oy = b.OB + nc;
  const T* Oz = b.OB + 2 * nc;
  const int wlo = a.wind_lo, wn = a.wind ? a.wind_n : 0;
  const long long wn3 = (long long)wn * wn * wn;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(c, n, &i, &j, &k);
    auto D6 = [&](const T* g, int ax) {
      return fd6(g[nb(i, j, k, ax, -3, n)], g[nb(i, j, k, ax, -2, n)], g[nb(i, j, k, ax, -1, n)], g[c],
                 g[nb(i, j, k, ax, 1, n)], g[nb(i, j, k, ax, 2, n)]);
    };
    T rb[3];
    rb[0] = -dtdx * D6(Oz, 1) + dtdx * D6(Oy, 2);
    rb[1] = -dtdx * D6(Ox, 2) + dtdx * D6(Oz, 0);
    rb[2] = -dtdx * D6(Oy, 0) + dtdx * D6(Ox, 1);
    // the wind source of this stage (k_wind_source), for the cells of the taper's cube
    T ws[5] = {T(0), T(0), T(0), T(0), T(0)};
    const unsigned wi = (unsigned)(i - wlo), wj = (unsigned)(j - wlo), wk = (unsigned)(k - wlo);
    const bool wind = wi < (unsigned)wn && wj < (unsigned)wn && wk < (unsigned)wn;
    if (wind) {
      const long long w = ((long long)wi * wn + wj) * wn + wk;
#pragma unroll
      for (int r = 0; r < 5; ++r) ws[r] = b.WS[r * wn3 + w];
    }
    auto rhs = [&](int r) {
      const T rq = -dtdx * b.ACC[r * nc + c];
      return (wind && r < 5) ? rq + ws[r] : rq;
    };
    if (stage < 4) {
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const T rq = rhs(r);
        const T q = k0 * b.Q0[r * nc + c] + kc * b.Q[r * nc + c] + rq;
        b.Q[r * nc + c] = q;
        b.QF[r * nc + c] = b.QF[r * nc + c] + q * f;
      }
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const T bn = k0 * b0[r * nc + c] + kc * bcur[r * nc + c] + rb[r];
        b.B[r * nc + c] = bn;
        b.BF[r * nc + c] = b.BF[r * nc + c] + bn * f;
      }
    } else {
#pragma unroll
      for (int r = 0; r < 8; ++r) b.QF[r * nc + c] = b.QF[r * nc + c] + rhs(r);
#pragma unroll
      for (int r = 0; r < 3; ++r) b.BF[r * nc + c] = b.BF[r * nc + c] + rb[r];
    }
  }
}

// q_final -> primitives, faces -> state; advances t (last block)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_finalize(Bufs<T> b) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const FDArgs a = b.a;
  const T gamma = T(a.gamma), rhomin = T(a.rhomin), pgmin = T(a.pgmin);
  const int n = a.n;
  const long long nc = a.nc;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(c, n, &i, &j, &k);
    T U[8], P[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) U[r] = b.QF[r * nc + c];
    ucc(U, b.BF, b.BF + nc, b.BF + 2 * nc, i, j, k, n);
    if (a.enforce_positivity) positivity(U, gamma, rhomin, pgmin);
    cons_to_prim(U, P, gamma, rhomin, pgmin, a.enforce_positivity != 0);
#pragma unroll
    for (int r = 0; r < 8; ++r) b.P[r * nc + c] = P[r];
#pragma unroll
    for (int r = 0; r < 3; ++r) b.P[(8 + r) * nc + c] = b.BF[r * nc + c];
  }
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(&b.ctl->done_count, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    b.ctl->t = b.ctl->t + b.ctl->dt;
    b.ctl->steps = b.ctl->steps + 1;
    b.ctl->done_count = 0u;
    __threadfence();
  }
}


// ---------------------------------------------------------------- typed launchers


template <typename T>
Bufs<T> make_bufs(const FDLaunch& L, void* state, const FDArgs& a) {
  Bufs<T> b;
  b.P = static_cast<T*>(state);
  T** dst[10] = {&b.Q0, &b.Q, &b.QF, &b.QC, &b.ACC, &b.B, &b.BF, &b.M, &b.OM, &b.OB};
  for (int i = 0; i < 10; ++i) *dst[i] = static_cast<T*>(L.bufs[i]);
  b.ctl = L.ctl;
  b.WS = static_cast<T*>(L.wind_src);
  b.a = a;
  return b;
}

template <typename T>
int set_attrs() {
  const int smem = (int)weno_smem<T>();
  int rc = cudaFuncSetAttribute(k_weno<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess;
  rc |= cudaFuncSetAttribute(k_weno<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess;
  rc |= cudaFuncSetAttribute(k_weno<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess;
  return rc ? AMX_ERR_CUDA : AMX_OK;
}

// one step without the CFL reduction (dt already in the control block)
template <typename T>
int launch_stages(const FDLaunch& L, void* state, const FDArgs& a, cudaStream_t s) {
  Bufs<T> b = make_bufs<T>(L, state, a);
  const int g = L.grid;
  const int n = L.n;
  constexpr int kA = WenoTile<T>::A, kL = WenoTile<T>::L;
  const dim3 wg((n + kA - 1) / kA, (n + kL - 1) / kL, n);
  const size_t wsm = weno_smem<T>();
  for (int st = 0; st < 5; ++st) {
    k_prep<T><<<g, kThreads, 0, s>>>(b, st);
    k_weno<T, 0><<<wg, kThreads, wsm, s>>>(b);
    k_weno<T, 1><<<wg, kThreads, wsm, s>>>(b);
    k_weno<T, 2><<<wg, kThreads, wsm, s>>>(b);
    k_emf<T><<<g, kThreads, 0, s>>>(b);
    k_emf_avg<T><<<g, kThreads, 0, s>>>(b);
    if (a.wind) {
      const long long wn3 = (long long)a.wind_n * a.wind_n * a.wind_n;
      const int wg = (int)((wn3 + kThreads - 1) / kThreads < g ? (wn3 + kThreads - 1) / kThreads : g);
      k_wind_source<T><<<wg, kThreads, 0, s>>>(b, st);
    }
    k_update<T><<<g, kThreads, 0, s>>>(b, st);
  }
  k_finalize<T><<<g, kThreads, 0, s>>>(b);
  return cudaGetLastError() == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
}

template <typename T>
int launch_cfl(const FDLaunch& L, const void* state, const FDArgs& a, cudaStream_t s) {
  Bufs<T> b = make_bufs<T>(L, const_cast<void*>(state), a);
  k_cfl<T><<<L.grid, kThreads, 0, s>>>(b);
  return cudaGetLastError() == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
}

#define AMX_FD_INSTANTIATE(T, SUFFIX)                                                                 \
  int fd_set_attrs_##SUFFIX() { return set_attrs<T>(); }                                             \
  int fd_launch_stages_##SUFFIX(const FDLaunch& L, void* st, const FDArgs& a, cudaStream_t s) {      \
    return launch_stages<T>(L, st, a, s);                                                            \
  }                                                                                                  \
  int fd_launch_cfl_##SUFFIX(const FDLaunch& L, const void* st, const FDArgs& a, cudaStream_t s) {   \
    return launch_cfl<T>(L, st, a, s);                                                               \
  }

}  // namespace fd
}  // namespace amx
