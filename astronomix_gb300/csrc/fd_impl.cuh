// Finite-difference WENO-CT MHD step: kernels and their typed launchers.
//
// One time step = 1 CFL reduction + 5 SSPRK(5,4) stages x 7 sweeps + 1
// finalize sweep + the time advance (38 launches), all stream-ordered, reading
// dt from the device control block (no host round trip per step).  Stage s:
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

// The pointwise sweeps run one thread per cell on a 3D grid: blocks of 32
// (z) x 8 (y) threads, grid (n/32, n/8, n) -- (i, j, k) come from the block
// and thread indices, with no integer division.
constexpr int kSweepZ = 32, kSweepY = 8;
inline dim3 sweep_grid(int n) { return dim3((n + kSweepZ - 1) / kSweepZ, (n + kSweepY - 1) / kSweepY, n); }
inline dim3 sweep_block() { return dim3(kSweepZ, kSweepY, 1); }
__device__ __forceinline__ bool sweep_cell(int n, int* i, int* j, int* k, long long* c) {
  *k = blockIdx.x * kSweepZ + threadIdx.x;
  *j = blockIdx.y * kSweepY + threadIdx.y;
  *i = blockIdx.z;
  if (*k >= n || *j >= n) return false;
  *c = cidx(*i, *j, *k, n);
  return true;
}
// Resident blocks per SM that the FP32 prep and EMF sweeps budget their
// registers for (AMX_FD_SWEEP_BLOCKS; latency-bound sweeps: more warps in
// flight).  256^3 ms per launch, prep / EMF / EMF average: 0.33 / 0.17 /
// 0.13 at the compiler's own budget, 0.31 / 0.15 / 0.12 at 6 blocks,
// 0.30 / 0.18 / 0.12 at 8 (spills in the EMF sweeps).
#ifndef AMX_FD_SWEEP_BLOCKS
#define AMX_FD_SWEEP_BLOCKS 6
#endif
// The EMF sweeps, whose stencils reach along x: a thread takes XW
// consecutive x cells of one (y, z) column, loads each x plane of an
// x-direction stencil once, and has XW cells' loads in flight.  (The face
// update and the prep stay at one cell a thread: 4 cells took the update
// from 48 to 80 registers and from 0.48 to 0.52 ms per 256^3 launch, the
// prep from 0.33 to 0.36 ms.)
constexpr int kSweepXEmf = 4;
template <int XW>
inline dim3 sweep_grid_x(int n) {
  return dim3((n + kSweepZ - 1) / kSweepZ, (n + kSweepY - 1) / kSweepY, (n + XW - 1) / XW);
}
template <int XW>
__device__ __forceinline__ bool sweep_column(int n, int* i0, int* j, int* k) {
  *k = blockIdx.x * kSweepZ + threadIdx.x;
  *j = blockIdx.y * kSweepY + threadIdx.y;
  *i0 = blockIdx.z * XW;
  return *k < n && *j < n;
}

template <typename T>
struct Bufs {
  T* P;    // state (prim, 11 rows)
  T* Q0;   // 8
  T* Q;    // 8
  T* QF;   // 8
  T* QC;   // 8
  T* ACC;  // 2 x 8: the flux differences of the y and z interfaces (the x pass, last, sums them)
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
      dt = nanmin(dt, a.dt_max);
      active = (t < a.t_end) ? 1 : 0;
    }
    if (!(t < a.t_pause)) active = 0;
    if (a.exact_end_time) dt = nanmin(dt, a.t_end - t);
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
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? AMX_FD_SWEEP_BLOCKS : 1) k_prep(Bufs<T> b, int stage) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const FDArgs a = b.a;
  const T gamma = T(a.gamma), rhomin = T(a.rhomin), pgmin = T(a.pgmin);
  const long long nc = a.nc;
  const int n = a.n;
  const T* faces = (stage == 0) ? b.P + 8 * nc : b.B;
  const T f0 = T(kFIN[0]);
  int i, j, k;
  long long c;
  if (sweep_cell(n, &i, &j, &k, &c)) {
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
    ucc(U, faces, faces + nc, faces + 2 * nc, i, j, k, n);
#pragma unroll
    for (int r = 0; r < 8; ++r) b.QC[r * nc + c] = U[r];
  }
}

// ---------------------------------------------------------------- WENO

// Staged per-cell values of a WENO tile, in the permuted frame (the flux
// axis is "x"): the conserved state, the x-flux without its Bx row (always
// zero), the inputs of the interface eigenvector blocks and the wave speeds.
enum : int {
  SV_U = 0,    // rho mx my mz E Bx By Bz
  SV_F = 8,    // F: rho mx my mz E By Bz (F[Bx] = 0)
  SV_EV = 15,  // floored rho, vx vy vz (unfloored rho), specific enthalpy
  SV_C = 20,   // fast, Alfven, slow speed
  kSV = 23
};

// index of a permuted-frame conserved row in the 7-vectors (Bx dropped):
// rho mx my mz E By Bz -> 0..6, Bx -> -1
__host__ __device__ constexpr int c7(int row) { return row < BX ? row : (row == BX ? -1 : row - 1); }

// Tile of A cells along the flux axis x 32 lanes across it.  Every staged
// cell (A + 6 with the halo of 3) costs a flux and an eigensystem; every
// thread owns whole interfaces.  FP32: 128 threads, three blocks per SM (168
// registers a thread, 62-70 KB of shared memory a block), so that one
// block's staging loads and stores overlap the others' arithmetic; A = 13
// for the y and z passes, 11 for the x pass, whose stage epilogue reads 40
// values a cell.  Measured on the 256^3 blast, WENO x / y / z ms per launch
// (bank-conflict-free layout): 1.71 / 1.40 / 1.42 with A = 11, 1.77 / 1.36 /
// 1.38 with A = 13, 1.94 / 1.48 / 1.50 with A = 9; with the earlier layout
// 1.50 / 1.49 / 1.60 (11, 128 threads, 3 blocks, before the x pass took the
// stage), 1.53 / 1.51 / 1.56 (23, 192, 2), 1.64 / 1.63 / 1.69 (47, 384, 1).
// FP64: A = 15, 256 threads, one block.
#ifndef AMX_WENO_A32
#define AMX_WENO_A32 11
#endif
#ifndef AMX_WENO_A32_YZ
#define AMX_WENO_A32_YZ 13
#endif
#ifndef AMX_WENO_T32
#define AMX_WENO_T32 128
#endif
#ifndef AMX_WENO_B32
#define AMX_WENO_B32 3
#endif
template <typename T, int D> struct WenoTile {
  static constexpr int A = sizeof(T) == 4 ? (D == 0 ? AMX_WENO_A32 : AMX_WENO_A32_YZ) : 15;
  static constexpr int THREADS = sizeof(T) == 4 ? AMX_WENO_T32 : 256;
  static constexpr int BLOCKS = sizeof(T) == 4 ? AMX_WENO_B32 : 1;  // resident blocks per SM
  static constexpr int L = 32;
  static constexpr int AH = A + 6;          // staged cells per lane: the pitch along the axis (odd)
  static constexpr int FP = (A + 1) | 1;    // pitch of a lane's interface fluxes (odd)
  static_assert(AH % 2 == 1, "the staged rows need an odd pitch");
};

// Shared memory of a tile.  FP64: kSV scalar rows.  FP32: the flux and the
// state component a characteristic projection pairs with it as 7 float2
// rows (F_c, U_c), then 9 scalar rows (Bx, the eigenvector-block inputs,
// the wave speeds): the same 23 values a cell, laid out for the paired FP32
// arithmetic.  Then the interface fluxes, 7 rows.  Every row is lane-major
// with an odd pitch along the axis: warps that step across lanes (the
// interface sweep, the x and y staging) and warps that step along the axis
// (the z staging) both hit 32 distinct banks, for 4- and 8-byte values.
template <typename T, int D>
constexpr size_t weno_smem() {
  using W = WenoTile<T, D>;
  return sizeof(T) * ((size_t)kSV * W::L * W::AH + (size_t)7 * W::L * W::FP);
}
constexpr int kSX = 9;  // FP32 scalar rows: 0 Bx, 1-5 eigenvector-block inputs, 6-8 cf ca cs

// Views of a tile's staged cells in either layout.
template <typename T> struct WenoStage;
template <> struct WenoStage<double> {
  double* S;
  int AP, NL;  // pitch along the axis, lanes
  __device__ double& v(int row, int ai, int li) const { return S[((size_t)row * NL + li) * AP + ai]; }
  __device__ void store(const double* out, int ai, int li) const {
#pragma unroll
    for (int k = 0; k < kSV; ++k) v(k, ai, li) = out[k];
  }
  __device__ double U(int r, int ai, int li) const { return v(SV_U + r, ai, li); }
  __device__ double F(int c, int ai, int li) const { return v(SV_F + c, ai, li); }
  __device__ double EV(int k, int ai, int li) const { return v(SV_EV + k, ai, li); }
  __device__ double C(int k, int ai, int li) const { return v(SV_C + k, ai, li); }
};
template <> struct WenoStage<float> {
  float2* P;  // [7][lanes][AP] (F_c, U_c)
  float* X;   // [kSX][lanes][AP]
  int AP, NL;  // pitch along the axis, lanes
  __device__ float2& p(int c, int ai, int li) const { return P[((size_t)c * NL + li) * AP + ai]; }
  __device__ float& x(int k, int ai, int li) const { return X[((size_t)k * NL + li) * AP + ai]; }
  __device__ void store(const float* out, int ai, int li) const {
#pragma unroll
    for (int c = 0; c < 7; ++c) p(c, ai, li) = make_float2(out[SV_F + c], out[SV_U + (c < 5 ? c : c + 1)]);
    x(0, ai, li) = out[SV_U + BX];
#pragma unroll
    for (int k = 0; k < 5; ++k) x(1 + k, ai, li) = out[SV_EV + k];
#pragma unroll
    for (int k = 0; k < 3; ++k) x(6 + k, ai, li) = out[SV_C + k];
  }
  __device__ float U(int r, int ai, int li) const { return r == BX ? x(0, ai, li) : p(c7(r), ai, li).y; }
  __device__ float F(int c, int ai, int li) const { return p(c, ai, li).x; }
  __device__ float EV(int k, int ai, int li) const { return x(1 + k, ai, li); }
  __device__ float C(int k, int ai, int li) const { return x(6 + k, ai, li); }
};

// g mod n for g in [-n, n + span): a few compares instead of an integer
// division (the tiles' halo reaches 3 cells below 0 and A + 2 above n - 1)
__device__ __forceinline__ int pmod(int g, int n) {
  if (g < 0) g += n;
  while (g >= n) g -= n;
  return g;
}


// Everything a staged cell needs, with the arithmetic of _mhd_flux_x
// (_fluxes.py:23-69 via primitive_state_from_conserved), of the per-cell
// part of _eigenvector_building_blocks (_eigen.py:124-162) and of
// _eigenvalue_building_blocks (_eigen.py:28-114), sharing the velocities.
template <typename T>
__device__ __forceinline__ void weno_cell(const T* U, T gamma, T rhomin, T pgmin, bool floors, T* out) {
  const T rho = U[RHO];
  const T vx = U[MX] / rho, vy = U[MY] / rho, vz = U[MZ] / rho;
  const T Bx = U[BX], By = U[BY], Bz = U[BZ];
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T b2 = Bx * Bx + By * By + Bz * Bz;
  // flux (primitive_state_from_conserved_mhd, optional floors)
  {
    T p = (gamma - T(1)) * (U[EN] - T(0.5) * rho * v2 - T(0.5) * b2);
    T rf = rho;
    if (floors) {
      rf = jmax(rho, rhomin);
      p = jmax(p, pgmin);
    }
    const T ptot = p + T(0.5) * b2;
    const T vdotB = vx * Bx + vy * By + vz * Bz;
    const T E = p / (gamma - T(1)) + T(0.5) * rf * v2 + T(0.5) * b2;
    out[SV_F + 0] = rf * vx;
    out[SV_F + 1] = rf * (vx * vx) + ptot - Bx * Bx;
    out[SV_F + 2] = rf * vx * vy - Bx * By;
    out[SV_F + 3] = rf * vx * vz - Bx * Bz;
    out[SV_F + 4] = (E + ptot) * vx - vdotB * Bx;
    out[SV_F + 5] = By * vx - Bx * vy;
    out[SV_F + 6] = Bz * vx - Bx * vz;
  }
  // eigen building blocks (floors always, _eigen.py:61-74 and :140-150)
  // (each jnp.where re-tests its condition on the values already floored)
  T pg = (gamma - T(1)) * (U[EN] - T(0.5) * (rho * v2 + b2));
  const T r = ((rho < rhomin) || (pg < pgmin)) ? jmax(rho, rhomin) : rho;
  pg = ((r < rhomin) || (pg < pgmin)) ? jmax(pg, pgmin) : pg;
  const T energy = ((r < rhomin) || (pg < pgmin)) ? pg / (gamma - T(1)) + T(0.5) * (r * v2 + b2) : U[EN];
  out[SV_EV + 0] = r;
  out[SV_EV + 1] = vx;
  out[SV_EV + 2] = vy;
  out[SV_EV + 3] = vz;
  out[SV_EV + 4] = (energy + pg) / r;
  const T cs2 = jmax(T(0), gamma * Num<T>::abs_(pg / r));
  const T b2r = b2 / r;
  const T disc = dss(jmax(T(0), sq(b2r + cs2) - T(4) * (Bx * Bx) / r * cs2));
  out[SV_C + 0] = dss(jmax(T(0), T(0.5) * (b2r + cs2 + disc)));
  out[SV_C + 1] = dss(jmax(T(0), (Bx * Bx) / r));
  out[SV_C + 2] = dss(jmax(T(0), T(0.5) * (b2r + cs2 - disc)));
#pragma unroll
  for (int k = 0; k < 8; ++k) out[SV_U + k] = U[k];
}

// Left eigenvector row S (_eigen.py:677-909) in the 7-vector layout, times
// the 1/2 of the WENO inputs (_weno.py:185-188): an exact power-of-two
// scaling, so the projections equal the reference's halved.
template <typename T, int S>
__device__ __forceinline__ void L7(const EigIF<T>& e, T* L) {
  const T vx = e.vx, vy = e.vy, vz = e.vz, vsq = e.vsq, bty = e.bty, btz = e.btz, sbx = e.sbx;
  const T a = e.a, cf = e.cf, cs = e.cs, af = e.af, aS = e.as, sr = e.sr;
  const T gam0 = e.gam0, gam1 = e.gam1;
  if constexpr (S == 0 || S == 6) {
    // 0.5 L a2inv (x sbt when a < ca), halved: exact scalings of one product
    const T q = (e.ge ? T(0.25) : T(0.25) * e.sbt) * e.a2inv;
    if constexpr (S == 0) {
      L[0] = af * (gam1 * vsq + cf * vx) - aS * cs * (bty * vy + btz * vz) * sbx;
      L[1] = af * (gam0 * vx - cf);
      L[2] = gam0 * af * vy + aS * cs * bty * sbx;
      L[3] = gam0 * af * vz + aS * cs * btz * sbx;
    } else {
      L[0] = af * (gam1 * vsq - cf * vx) + aS * cs * (bty * vy + btz * vz) * sbx;
      L[1] = af * (gam0 * vx + cf);
      L[2] = gam0 * af * vy - aS * cs * bty * sbx;
      L[3] = gam0 * af * vz - aS * cs * btz * sbx;
    }
    L[4] = -gam0 * af;
    L[5] = gam0 * af * e.by + a * aS * bty * sr;
    L[6] = gam0 * af * e.bz + a * aS * btz * sr;
#pragma unroll
    for (int k = 0; k < 7; ++k) L[k] = L[k] * q;
  } else if constexpr (S == 2 || S == 4) {
    const T q = (e.ge ? T(0.25) * e.sbt : T(0.25)) * e.a2inv;
    if constexpr (S == 2) {
      L[0] = aS * (gam1 * vsq + cs * vx) + af * cf * (bty * vy + btz * vz) * sbx;
      L[1] = gam0 * aS * vx - aS * cs;
      L[2] = gam0 * aS * vy - af * cf * bty * sbx;
      L[3] = gam0 * aS * vz - af * cf * btz * sbx;
    } else {
      L[0] = aS * (gam1 * vsq - cs * vx) - af * cf * (bty * vy + btz * vz) * sbx;
      L[1] = aS * (gam0 * vx + cs);
      L[2] = gam0 * aS * vy + af * cf * bty * sbx;
      L[3] = gam0 * aS * vz + af * cf * btz * sbx;
    }
    L[4] = -gam0 * aS;
    L[5] = gam0 * aS * e.by - a * af * bty * sr;
    L[6] = gam0 * aS * e.bz - a * af * btz * sr;
#pragma unroll
    for (int k = 0; k < 7; ++k) L[k] = L[k] * q;
  } else if constexpr (S == 1 || S == 5) {
    L[0] = T(0.25) * (btz * vy - bty * vz);
    L[1] = T(0);
    L[2] = T(0.25) * (-btz);
    L[3] = T(0.25) * bty;
    L[4] = T(0);
    if constexpr (S == 1) {
      L[5] = T(0.25) * (-btz * sbx * sr);
      L[6] = T(0.25) * (bty * sbx * sr);
    } else {
      L[5] = T(0.25) * (btz * sbx * sr);
      L[6] = T(0.25) * (-bty * sbx * sr);
    }
  } else {  // 3: entropy, -gam0 L a2inv, halved
    const T q = T(0.5) * e.a2inv;
    L[0] = -gam0 * (-e.a2 / gam0 - T(0.5) * vsq) * q;
    L[1] = -gam0 * vx * q;
    L[2] = -gam0 * vy * q;
    L[3] = -gam0 * vz * q;
    L[4] = -gam0 * T(-1) * q;
    L[5] = -gam0 * e.by * q;
    L[6] = -gam0 * e.bz * q;
  }
}

// Right eigenvector column S (_eigen.py:392-620) in the 7-vector layout.
template <typename T, int S>
__device__ __forceinline__ void R7(const EigIF<T>& e, T* R) {
  const T vx = e.vx, vy = e.vy, vz = e.vz, vsq = e.vsq, bty = e.bty, btz = e.btz, sbx = e.sbx;
  const T a = e.a, a2 = e.a2, cf = e.cf, cs = e.cs, af = e.af, aS = e.as, sr = e.sr, gam2 = e.gam2;
  if constexpr (S == 0) {
    R[0] = af;
    R[1] = af * (vx - cf);
    R[2] = af * vy + aS * cs * bty * sbx;
    R[3] = af * vz + aS * cs * btz * sbx;
    R[4] = af * (cf * cf - cf * vx + T(0.5) * vsq - gam2 * a2) + aS * cs * (bty * vy + btz * vz) * sbx;
    R[5] = a * aS * bty / sr;
    R[6] = a * aS * btz / sr;
  } else if constexpr (S == 6) {
    R[0] = af;
    R[1] = af * (vx + cf);
    R[2] = af * vy - aS * cs * bty * sbx;
    R[3] = af * vz - aS * cs * btz * sbx;
    R[4] = af * (cf * cf + cf * vx + T(0.5) * vsq - gam2 * a2) - aS * cs * (bty * vy + btz * vz) * sbx;
    R[5] = a * aS * bty / sr;
    R[6] = a * aS * btz / sr;
  } else if constexpr (S == 2) {
    R[0] = aS;
    R[1] = aS * (vx - cs);
    R[2] = aS * vy - af * cf * bty * sbx;
    R[3] = aS * vz - af * cf * btz * sbx;
    R[4] = aS * (cs * cs - cs * vx + T(0.5) * vsq - gam2 * a2) - af * cf * (bty * vy + btz * vz) * sbx;
    R[5] = -a * af * bty / sr;
    R[6] = -a * af * btz / sr;
  } else if constexpr (S == 4) {
    R[0] = aS;
    R[1] = aS * (vx + cs);
    R[2] = aS * vy + af * cf * bty * sbx;
    R[3] = aS * vz + af * cf * btz * sbx;
    R[4] = aS * (cs * cs + cs * vx + T(0.5) * vsq - gam2 * a2) + af * cf * (bty * vy + btz * vz) * sbx;
    R[5] = -a * af * bty / sr;
    R[6] = -a * af * btz / sr;
  } else if constexpr (S == 1 || S == 5) {
    R[0] = T(0);
    R[1] = T(0);
    R[2] = -btz;
    R[3] = bty;
    R[4] = bty * vz - btz * vy;
    if constexpr (S == 1) {
      R[5] = -btz * sbx / sr;
      R[6] = bty * sbx / sr;
    } else {
      R[5] = btz * sbx / sr;
      R[6] = -bty * sbx / sr;
    }
  } else {  // 3
    R[0] = T(1);
    R[1] = vx;
    R[2] = vy;
    R[3] = vz;
    R[4] = T(0.5) * vsq;
    R[5] = T(0);
    R[6] = T(0);
  }
  // fast modes flip when a < ca, slow modes when a >= ca
  if constexpr (S == 0 || S == 6 || S == 2 || S == 4) {
    const bool flip = (S == 0 || S == 6) ? !e.ge : e.ge;
    if (flip) {
#pragma unroll
      for (int k = 0; k < 7; ++k) R[k] = R[k] * e.sbt;
    }
  }
}

// Nonzero entries of the rows and columns: the Alfven rows have no mx and E
// entries, the Alfven columns no rho and mx, the entropy column no B.
template <int S> __host__ __device__ constexpr unsigned lmask() { return (S == 1 || S == 5) ? 0x6Du : 0x7Fu; }
template <int S> __host__ __device__ constexpr unsigned rmask() {
  return (S == 1 || S == 5) ? 0x7Cu : (S == 3 ? 0x1Fu : 0x7Fu);
}

// One characteristic field of _weno.py:136-238 at one interface: project the
// five flux and state differences of the stencil (dF[k] = F[i-1+k] -
// F[i-2+k]), LF-split with alpha_s, WENO-weight both sides and add
// R_s (third - second) to the interface flux.
template <typename T, int S>
__device__ __forceinline__ void weno_mode(const EigIF<T>& e, const T (&dF)[5][7], const T (&dq)[5][7], T alpha,
                                          T (&Fi)[7]) {
  constexpr unsigned LM = lmask<S>(), RM = rmask<S>();
  T L[7];
  L7<T, S>(e, L);
  T d[5], q[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    T sd = T(0), sq_ = T(0);
    bool first = true;
#pragma unroll
    for (int c = 0; c < 7; ++c) {
      if (LM & (1u << c)) {
        if (first) {
          sd = L[c] * dF[k][c];
          sq_ = L[c] * dq[k][c];
          first = false;
        } else {
          sd = sd + L[c] * dF[k][c];
          sq_ = sq_ + L[c] * dq[k][c];
        }
      }
    }
    d[k] = sd;
    q[k] = sq_;
  }
  const T second = weno_phi(d[0] + alpha * q[0], d[1] + alpha * q[1], d[2] + alpha * q[2], d[3] + alpha * q[3]);
  const T third = weno_phi(d[4] - alpha * q[4], d[3] - alpha * q[3], d[2] - alpha * q[2], d[1] - alpha * q[1]);
  const T Fs = -second + third;
  T R[7];
  R7<T, S>(e, R);
#pragma unroll
  for (int c = 0; c < 7; ++c)
    if (RM & (1u << c)) Fi[c] = Fi[c] + R[c] * Fs;
}

// ---- paired FP32 arithmetic (fma.rn.f32x2 and friends on sm_100+): two
// FP32 operations per issue slot, each rounded like its scalar form

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {  // a - b, exactly as two FSUBs
  return __ffma2_rn(b, f2(-1.f, -1.f), a);
}

// The two WENO interpolants of one characteristic field, weno_phi of
// (second, third) as one pair (_weno.py:186-228).
__device__ __forceinline__ float2 weno_phi2(float2 a, float2 b, float2 c, float2 d) {
  const float2 k13 = f2(13.f, 13.f), k3 = f2(3.f, 3.f), eps = f2(1e-8f, 1e-8f);
  const float2 t0 = f2sub(a, b), u0 = __ffma2_rn(b, f2(-3.f, -3.f), a);
  const float2 IS0 = __ffma2_rn(k13, __fmul2_rn(t0, t0), __fmul2_rn(k3, __fmul2_rn(u0, u0)));
  const float2 t1 = f2sub(b, c), u1 = __fadd2_rn(b, c);
  const float2 IS1 = __ffma2_rn(k13, __fmul2_rn(t1, t1), __fmul2_rn(k3, __fmul2_rn(u1, u1)));
  const float2 t2 = f2sub(c, d), u2 = __ffma2_rn(c, k3, f2(-d.x, -d.y));
  const float2 IS2 = __ffma2_rn(k13, __fmul2_rn(t2, t2), __fmul2_rn(k3, __fmul2_rn(u2, u2)));
  const float2 e0 = __fadd2_rn(eps, IS0), e1 = __fadd2_rn(eps, IS1), e2 = __fadd2_rn(eps, IS2);
  const float2 s0 = __fmul2_rn(e0, e0), s1 = __fmul2_rn(e1, e1), s2 = __fmul2_rn(e2, e2);
  const float2 al0 = f2(1.f / s0.x, 1.f / s0.y);
  const float2 al1 = __fmul2_rn(f2(6.f, 6.f), f2(1.f / s1.x, 1.f / s1.y));
  const float2 al2 = __fmul2_rn(k3, f2(1.f / s2.x, 1.f / s2.y));
  float2 asum = __fadd2_rn(__fadd2_rn(al0, al1), al2);
  asum = f2(fmaxf(asum.x, 1e-14f), fmaxf(asum.y, 1e-14f));
  const float2 r = f2(1.f / asum.x, 1.f / asum.y);
  const float2 w0 = __fmul2_rn(al0, r), w2 = __fmul2_rn(al2, r);
  const float2 p = __fadd2_rn(__ffma2_rn(b, f2(-2.f, -2.f), a), c);
  const float2 q = __fadd2_rn(__ffma2_rn(c, f2(-2.f, -2.f), b), d);
  const float2 first = __fmul2_rn(__fmul2_rn(w0, p), f2(1.f / 3.f, 1.f / 3.f));
  const float2 g = __fmul2_rn(__fadd2_rn(w2, f2(-0.5f, -0.5f)), q);
  return __ffma2_rn(g, f2(1.f / 6.f, 1.f / 6.f), first);
}

// One characteristic field (weno_mode) with the stencil differences held as
// (flux, state) pairs: each left-row coefficient multiplies both at once.
template <int S>
__device__ __forceinline__ void weno_mode2(const EigIF<float>& e, const float2 (&dd)[5][7], float alpha,
                                           float (&Fi)[7]) {
  constexpr unsigned LM = lmask<S>(), RM = rmask<S>();
  float L[7];
  L7<float, S>(e, L);
  float2 dq[5];  // (L.dF_k, L.dq_k), halved
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    float2 acc = f2(0.f, 0.f);
    bool first = true;
#pragma unroll
    for (int c = 0; c < 7; ++c) {
      if (LM & (1u << c)) {
        const float2 l = f2(L[c], L[c]);
        acc = first ? __fmul2_rn(dd[k][c], l) : __ffma2_rn(dd[k][c], l, acc);
        first = false;
      }
    }
    dq[k] = acc;
  }
  // inputs of the two interpolants: second (d_k + alpha q_k, k = 0..3),
  // third (d_k - alpha q_k, k = 4..1), interleaved as pairs
  const float2 A = f2(fmaf(alpha, dq[0].y, dq[0].x), fmaf(-alpha, dq[4].y, dq[4].x));
  const float2 B = f2(fmaf(alpha, dq[1].y, dq[1].x), fmaf(-alpha, dq[3].y, dq[3].x));
  const float2 C = f2(fmaf(alpha, dq[2].y, dq[2].x), fmaf(-alpha, dq[2].y, dq[2].x));
  const float2 D = f2(fmaf(alpha, dq[3].y, dq[3].x), fmaf(-alpha, dq[1].y, dq[1].x));
  const float2 st = weno_phi2(A, B, C, D);
  const float Fs = -st.x + st.y;
  float R[7];
  R7<float, S>(e, R);
#pragma unroll
  for (int c = 0; c < 7; ++c)
    if (RM & (1u << c)) Fi[c] = Fi[c] + R[c] * Fs;
}

// Interface fluxes along axis D (0 = x, 1 = y, 2 = z), _weno.py:112-324,
// with the CT-corrected fluxes of the two tangential field components
// (_constrained_transport.py:77-102) fused into the store.  The z and y
// passes run first and store their flux differences; the x pass, whose lanes
// run along the contiguous z axis, adds its own to theirs and applies the
// stage: the right-hand side of the cell-centred rows and the SSPRK(5,4)
// combination (_ssprk.py:224-228, :298-310, :328-332).  The face fields are
// k_update's, after the EMFs.
template <typename T, int D>
__global__ void __launch_bounds__(WenoTile<T, D>::THREADS, WenoTile<T, D>::BLOCKS) k_weno(Bufs<T> b, int stage) {
  using W = WenoTile<T, D>;
  constexpr int kA = W::A, kL = W::L, kFP = W::FP, kAH = W::AH, kT = W::THREADS;
  FD_ACTIVE_OR_RETURN(b.ctl);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WenoStage<T> st;
  T* FI;  // [7][kL][kFP] (permuted frame)
  if constexpr (sizeof(T) == 4) {
    st.P = reinterpret_cast<float2*>(smem_raw);
    st.X = reinterpret_cast<float*>(st.P + (size_t)7 * kL * kAH);
    FI = st.X + (size_t)kSX * kL * kAH;
  } else {
    st.S = reinterpret_cast<T*>(smem_raw);
    FI = st.S + (size_t)kSV * kL * kAH;
  }
  st.AP = kAH;
  st.NL = kL;
  auto fi = [&](int c, int ii, int li) -> T& { return FI[((size_t)c * kL + li) * kFP + ii]; };
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

  // ---- stage the cells a0-3 .. a0+kA+2 (permuted frame); the z tile walks
  // along z within a warp so that its loads stay coalesced
  for (int e = threadIdx.x; e < kAH * kL; e += kT) {
    int ai, li;
    if (D == 2) { ai = e % kAH; li = e / kAH; }
    else { li = e % kL; ai = e / kL; }
    const int ga = pmod(a0 - 3 + ai, n);
    int gl = l0 + li;
    if (gl >= n) gl = n - 1;
    const long long c = cell_of(ga, gl);
    T U[8], out[kSV];
#pragma unroll
    for (int r = 0; r < 8; ++r) U[r] = b.QC[perm_row(D, r) * nc + c];
    weno_cell(U, gamma, rhomin, pgmin, floors, out);
    st.store(out, ai, li);
  }
  __syncthreads();

  // ---- interfaces a0-1 .. a0+kA-1 (local ii = 0..kA): cell i = a0-1+ii is
  // staged row ii+2, its stencil i-2 .. i+3 rows ii .. ii+5
#pragma unroll 1
  for (int task = threadIdx.x; task < (kA + 1) * kL; task += kT) {
    const int li = task % kL, ii = task / kL;
    // alpha_s = max |lambda_s| over the six stencil cells (cell centred)
    T al[7];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const T vx = st.EV(1, ii + m, li), cf = st.C(0, ii + m, li), ca = st.C(1, ii + m, li),
              cs = st.C(2, ii + m, li);
      const T lam[7] = {vx - cf, vx - ca, vx - cs, vx, vx + cs, vx + ca, vx + cf};
#pragma unroll
      for (int s = 0; s < 7; ++s) al[s] = (m == 0) ? Num<T>::abs_(lam[s]) : wmax(al[s], Num<T>::abs_(lam[s]));
    }
    // eigenvector blocks from cells i (row ii+2) and i+1 (row ii+3)
    EigIF<T> e;
    {
      T cL[5], cR[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        cL[k] = st.EV(k, ii + 2, li);
        cR[k] = st.EV(k, ii + 3, li);
      }
      eig_interface(cL, cR, st.U(BX, ii + 2, li), st.U(BY, ii + 2, li), st.U(BZ, ii + 2, li), st.U(BX, ii + 3, li),
                    st.U(BY, ii + 3, li), st.U(BZ, ii + 3, li), gamma, e);
    }
    // the base flux 1/12 (-F[i-1] + 7 F[i] + 7 F[i+1] - F[i+2]) and the
    // differences of the flux and the state over the stencil
    T Fi[7];
#pragma unroll
    for (int c = 0; c < 7; ++c)
      Fi[c] = T(1.0 / 12.0) * (-st.F(c, ii + 1, li) + T(7) * st.F(c, ii + 2, li) + T(7) * st.F(c, ii + 3, li) -
                               st.F(c, ii + 4, li));
    if constexpr (sizeof(T) == 4) {
      float2 dd[5][7];  // (F[m+1] - F[m], U[m+1] - U[m])
#pragma unroll
      for (int c = 0; c < 7; ++c) {
        float2 prev = st.p(c, ii, li);
#pragma unroll
        for (int m = 1; m < 6; ++m) {
          const float2 cur = st.p(c, ii + m, li);
          dd[m - 1][c] = f2sub(cur, prev);
          prev = cur;
        }
      }
      weno_mode2<0>(e, dd, al[0], Fi);
      weno_mode2<1>(e, dd, al[1], Fi);
      weno_mode2<2>(e, dd, al[2], Fi);
      weno_mode2<3>(e, dd, al[3], Fi);
      weno_mode2<4>(e, dd, al[4], Fi);
      weno_mode2<5>(e, dd, al[5], Fi);
      weno_mode2<6>(e, dd, al[6], Fi);
    } else {
      T dF[5][7], dq[5][7];
#pragma unroll
      for (int c = 0; c < 7; ++c) {
        const int r = c < 5 ? c : c + 1;
        T fp = st.F(c, ii, li), qp = st.U(r, ii, li);
#pragma unroll
        for (int m = 1; m < 6; ++m) {
          const T f = st.F(c, ii + m, li), q = st.U(r, ii + m, li);
          dF[m - 1][c] = f - fp;
          dq[m - 1][c] = q - qp;
          fp = f;
          qp = q;
        }
      }
      weno_mode<T, 0>(e, dF, dq, al[0], Fi);
      weno_mode<T, 1>(e, dF, dq, al[1], Fi);
      weno_mode<T, 2>(e, dF, dq, al[2], Fi);
      weno_mode<T, 3>(e, dF, dq, al[3], Fi);
      weno_mode<T, 4>(e, dF, dq, al[4], Fi);
      weno_mode<T, 5>(e, dF, dq, al[5], Fi);
      weno_mode<T, 6>(e, dF, dq, al[6], Fi);
    }
#pragma unroll
    for (int c = 0; c < 7; ++c) fi(c, ii, li) = Fi[c];
  }
  __syncthreads();

  // ---- cells a0 .. a0+kA-1: the flux difference of this axis (stored by
  // the z and y passes; the x pass applies the stage), the CT-corrected
  // fluxes at their faces
  // lab rows of the two tangential B components whose fluxes CT corrects
  constexpr int T1 = (D == 0) ? BY : BX;
  constexpr int T2 = (D == 2) ? BY : BZ;
  T* const acc = b.ACC + (size_t)(D == 0 ? 0 : D - 1) * 8 * nc;
  // the x pass: stage constants and the stellar-wind cube
  const T dt = (D == 0) ? T(*(volatile double*)&b.ctl->dt) : T(0);
  const T dtdx = T(kRHS[stage]) * dt / T(a.dx);
  const T k0 = T(kK0[stage]), kc = T(kKC[stage]);
  const T fin = (stage < 4) ? T(kFIN[stage + 1]) : T(0);
  const int wlo = a.wind_lo, wn = a.wind ? a.wind_n : 0;
  const long long wn3 = (long long)wn * wn * wn;
  for (int task = threadIdx.x; task < kA * kL; task += kT) {
    int ci, li;
    if (D == 2) { ci = task % kA; li = task / kA; }
    else { li = task % kL; ci = task / kL; }
    const int ga = a0 + ci, gl = l0 + li;
    if (ga >= n || gl >= n) continue;
    const long long c = cell_of(ga, gl);
    // face i+1/2 is local interface ci+1, face i-1/2 is ci
    if constexpr (D != 0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int k = c7(perm_row(D, r));
        if (k < 0) continue;  // the flux of B along its own axis vanishes (never read)
        acc[r * nc + c] = fi(k, ci + 1, li) - fi(k, ci, li);
      }
    } else {
      // cell (i, j, k) = (ga, t3, gl); the wind source of this stage
      // (k_wind_source) inside the taper's cube
      T ws[5] = {T(0), T(0), T(0), T(0), T(0)};
      const unsigned wi = (unsigned)(ga - wlo), wj = (unsigned)(t3 - wlo), wk = (unsigned)(gl - wlo);
      const bool wind = wi < (unsigned)wn && wj < (unsigned)wn && wk < (unsigned)wn;
      if (wind) {
        const long long w = ((long long)wi * wn + wj) * wn + wk;
#pragma unroll
        for (int r = 0; r < 5; ++r) ws[r] = b.WS[r * wn3 + w];
      }
      // every load of the cell first (about 40 in flight per thread: the
      // stores below may alias them for the compiler), then the arithmetic
      const T* ay = b.ACC;
      const T* az = b.ACC + 8 * nc;
      T vy[8], vz[8], v0[8], vq[8], vf[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        // B_a's own-axis difference is exactly zero and never stored
        vy[r] = (r != BY) ? ay[r * nc + c] : T(0);
        vz[r] = (r != BZ) ? az[r * nc + c] : T(0);
        vf[r] = b.QF[r * nc + c];
        v0[r] = (stage < 4) ? b.Q0[r * nc + c] : T(0);
        vq[r] = (stage < 4) ? b.Q[r * nc + c] : T(0);
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        // the flux differences summed in the reference's order, (x + y) + z
        T sum;
        if (r == BX) sum = vy[r] + vz[r];
        else {
          const T ax = fi(c7(r), ci + 1, li) - fi(c7(r), ci, li);
          if (r == BY) sum = ax + vz[r];
          else if (r == BZ) sum = ax + vy[r];
          else sum = (ax + vy[r]) + vz[r];
        }
        const T rq0 = -dtdx * sum;
        const T rq = (wind && r < 5) ? rq0 + ws[r] : rq0;
        if (stage < 4) {
          const T q = k0 * v0[r] + kc * vq[r] + rq;
          b.Q[r * nc + c] = q;
          b.QF[r * nc + c] = vf[r] + q * fin;
        } else {
          b.QF[r * nc + c] = vf[r] + rq;
        }
      }
    }
    // c2f over cells i-1 .. i+2 (staged rows ci+2 .. ci+5) of B_d and v_t (lab frame)
    const T Bn = c2f(st.U(BX, ci + 2, li), st.U(BX, ci + 3, li), st.U(BX, ci + 4, li), st.U(BX, ci + 5, li));
    constexpr int m1 = perm_row_c(D, T1 - BX + MX) - MX, m2 = perm_row_c(D, T2 - BX + MX) - MX;
    const T v1 = c2f(st.EV(1 + m1, ci + 2, li), st.EV(1 + m1, ci + 3, li), st.EV(1 + m1, ci + 4, li),
                     st.EV(1 + m1, ci + 5, li));
    const T v2 = c2f(st.EV(1 + m2, ci + 2, li), st.EV(1 + m2, ci + 3, li), st.EV(1 + m2, ci + 4, li),
                     st.EV(1 + m2, ci + 5, li));
    b.M[(2 * D) * nc + c] = fi(c7(perm_row_c(D, T1)), ci + 1, li) + Bn * v1;
    b.M[(2 * D + 1) * nc + c] = fi(c7(perm_row_c(D, T2)), ci + 1, li) + Bn * v2;
  }
}

// ---------------------------------------------------------------- CT

// edge EMFs (_constrained_transport.py:104-131)
template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? AMX_FD_SWEEP_BLOCKS : 1) k_emf(Bufs<T> b) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const int n = b.a.n;
  const long long nc = b.a.nc;
  const T* By_fx = b.M;
  const T* Bz_fx = b.M + nc;
  const T* Bx_fy = b.M + 2 * nc;
  const T* Bz_fy = b.M + 3 * nc;
  const T* Bx_fz = b.M + 4 * nc;
  const T* By_fz = b.M + 5 * nc;
  int i0, j, k;
  if (sweep_column<kSweepXEmf>(n, &i0, &j, &k)) {
    // Bx_fy, Bx_fz at x = i0 - 1 + q (the x-direction interpolations)
    constexpr int WX = kSweepXEmf + 3;
    T wy[WX], wz[WX];
#pragma unroll
    for (int q = 0; q < WX; ++q) {
      const long long cq = cidx(wrap(i0 - 1 + q, n), j, k, n);
      wy[q] = Bx_fy[cq];
      wz[q] = Bx_fz[cq];
    }
#pragma unroll
    for (int u = 0; u < kSweepXEmf; ++u) {
      const int i = i0 + u;
      if (i >= n) break;
      const long long c = cidx(i, j, k, n);
      auto I = [&](const T* f, int ax) {
        return c2f(f[nb(i, j, k, ax, -1, n)], f[c], f[nb(i, j, k, ax, 1, n)], f[nb(i, j, k, ax, 2, n)]);
      };
      const T Oz = c2f(wy[u], wy[u + 1], wy[u + 2], wy[u + 3]) - I(By_fx, 1);
      const T Ox = I(By_fz, 1) - I(Bz_fy, 2);
      const T Oy = I(Bz_fx, 2) - c2f(wz[u], wz[u + 1], wz[u + 2], wz[u + 3]);
      b.OM[c] = Ox;
      b.OM[nc + c] = Oy;
      b.OM[2 * nc + c] = Oz;
    }
  }
}

// point values -> averages (_interpolate.py:39-62)
template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? AMX_FD_SWEEP_BLOCKS : 1) k_emf_avg(Bufs<T> b) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const int n = b.a.n;
  const long long nc = b.a.nc;
  int i0, j, k;
  if (sweep_column<kSweepXEmf>(n, &i0, &j, &k)) {
    // Omega_y, Omega_z at x = i0 - 1 + q (their x-direction second differences)
    constexpr int WX = kSweepXEmf + 2;
    T wy[WX], wz[WX];
#pragma unroll
    for (int q = 0; q < WX; ++q) {
      const long long cq = cidx(wrap(i0 - 1 + q, n), j, k, n);
      wy[q] = b.OM[nc + cq];
      wz[q] = b.OM[2 * nc + cq];
    }
#pragma unroll
    for (int u = 0; u < kSweepXEmf; ++u) {
      const int i = i0 + u;
      if (i >= n) break;
      const long long c = cidx(i, j, k, n);
      // q0 + (second difference along A) / 24 + (along B) / 24
      auto side = [&](const T* q, int B, T q0) {
        return (q[nb(i, j, k, B, -1, n)] - T(2) * q0 + q[nb(i, j, k, B, 1, n)]) / T(24);
      };
      auto xdiff = [&](const T* w, T q0) { return (w[u] - T(2) * q0 + w[u + 2]) / T(24); };
      const T ox = b.OM[c];
      b.OB[c] = ox + side(b.OM, 1, ox) + side(b.OM, 2, ox);                    // Omega_x: (y, z)
      b.OB[nc + c] = wy[u + 1] + xdiff(wy, wy[u + 1]) + side(b.OM + nc, 2, wy[u + 1]);   // Omega_y: (x, z)
      b.OB[2 * nc + c] = wz[u + 1] + xdiff(wz, wz[u + 1]) + side(b.OM + 2 * nc, 1, wz[u + 1]);  // Omega_z: (x, y)
    }
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
// (zero outside it), from the stage's input, before the x WENO pass adds it
// to the right-hand side.  Its own kernel, so that the FP64 arithmetic does
// not weigh on the WENO kernel's registers.
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

// The face fields' right-hand side (the EMF curl) and their SSPRK(5,4)
// combination (_ssprk.py:224-228, :298-310, :328-332); the cell-centred rows
// are the x WENO pass's.  Latency-bound (24 stencil loads a cell): in FP32
// the register budget is set for AMX_FD_UPDATE_BLOCKS resident blocks per SM
// (8: 32 registers, 0.53 -> 0.39 ms per 256^3 launch against the compiler's
// own 48 registers).
#ifndef AMX_FD_UPDATE_BLOCKS
#define AMX_FD_UPDATE_BLOCKS 8
#endif
template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? AMX_FD_UPDATE_BLOCKS : 1) k_update(Bufs<T> b, int stage) {
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
  int i, j, k;
  long long c;
  if (sweep_cell(n, &i, &j, &k, &c)) {
    auto D6 = [&](const T* g, int ax) {
      return fd6(g[nb(i, j, k, ax, -3, n)], g[nb(i, j, k, ax, -2, n)], g[nb(i, j, k, ax, -1, n)], g[c],
                 g[nb(i, j, k, ax, 1, n)], g[nb(i, j, k, ax, 2, n)]);
    };
    T rb[3];
    rb[0] = -dtdx * D6(Oz, 1) + dtdx * D6(Oy, 2);
    rb[1] = -dtdx * D6(Ox, 2) + dtdx * D6(Oz, 0);
    rb[2] = -dtdx * D6(Oy, 0) + dtdx * D6(Ox, 1);
    if (stage < 4) {
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const T bn = k0 * b0[r * nc + c] + kc * bcur[r * nc + c] + rb[r];
        b.B[r * nc + c] = bn;
        b.BF[r * nc + c] = b.BF[r * nc + c] + bn * f;
      }
    } else {
#pragma unroll
      for (int r = 0; r < 3; ++r) b.BF[r * nc + c] = b.BF[r * nc + c] + rb[r];
    }
  }
}

// q_final -> primitives, faces -> state (k_advance then advances t)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_finalize(Bufs<T> b) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  const FDArgs a = b.a;
  const T gamma = T(a.gamma), rhomin = T(a.rhomin), pgmin = T(a.pgmin);
  const int n = a.n;
  const long long nc = a.nc;
  int i, j, k;
  long long c;
  if (sweep_cell(n, &i, &j, &k, &c)) {
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
}

// the step's time advance, after k_finalize (one thread)
template <typename T>
__global__ void k_advance(Bufs<T> b) {
  FD_ACTIVE_OR_RETURN(b.ctl);
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    b.ctl->t = b.ctl->t + b.ctl->dt;
    b.ctl->steps = b.ctl->steps + 1;
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
  int rc = cudaFuncSetAttribute(k_weno<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)weno_smem<T, 0>()) !=
           cudaSuccess;
  rc |= cudaFuncSetAttribute(k_weno<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)weno_smem<T, 1>()) !=
        cudaSuccess;
  rc |= cudaFuncSetAttribute(k_weno<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)weno_smem<T, 2>()) !=
        cudaSuccess;
  return rc ? AMX_ERR_CUDA : AMX_OK;
}

// one step without the CFL reduction (dt already in the control block)
template <typename T>
int launch_stages(const FDLaunch& L, void* state, const FDArgs& a, cudaStream_t s) {
  Bufs<T> b = make_bufs<T>(L, state, a);
  const int g = L.grid;
  const int n = L.n;
  constexpr int kA = WenoTile<T, 0>::A, kAyz = WenoTile<T, 1>::A, kL = WenoTile<T, 0>::L;
  constexpr int kWT = WenoTile<T, 0>::THREADS;
  const dim3 wg((n + kA - 1) / kA, (n + kL - 1) / kL, n), wgyz((n + kAyz - 1) / kAyz, (n + kL - 1) / kL, n);
  const size_t wsm = weno_smem<T, 0>(), wsmyz = weno_smem<T, 1>();
  const dim3 g3 = sweep_grid(n), b3 = sweep_block();
  const dim3 gxe = sweep_grid_x<kSweepXEmf>(n);
  for (int st = 0; st < 5; ++st) {
    k_prep<T><<<g3, b3, 0, s>>>(b, st);
    fd_mark(L, FD_PH_PREP, s);
    if (a.wind) {  // from the stage's input (QC); the x pass adds it
      const long long wn3 = (long long)a.wind_n * a.wind_n * a.wind_n;
      const int wg = (int)((wn3 + kThreads - 1) / kThreads < g ? (wn3 + kThreads - 1) / kThreads : g);
      k_wind_source<T><<<wg, kThreads, 0, s>>>(b, st);
      fd_mark(L, FD_PH_WIND, s);
    }
    // z and y store their flux differences; x (last) applies the stage to Q
    k_weno<T, 2><<<wgyz, kWT, wsmyz, s>>>(b, st);
    fd_mark(L, FD_PH_WENO_Z, s);
    k_weno<T, 1><<<wgyz, kWT, wsmyz, s>>>(b, st);
    fd_mark(L, FD_PH_WENO_Y, s);
    k_weno<T, 0><<<wg, kWT, wsm, s>>>(b, st);
    fd_mark(L, FD_PH_WENO_X, s);
    k_emf<T><<<gxe, b3, 0, s>>>(b);
    fd_mark(L, FD_PH_EMF, s);
    k_emf_avg<T><<<gxe, b3, 0, s>>>(b);
    fd_mark(L, FD_PH_EMF_AVG, s);
    k_update<T><<<g3, b3, 0, s>>>(b, st);
    fd_mark(L, FD_PH_UPDATE, s);
  }
  k_finalize<T><<<g3, b3, 0, s>>>(b);
  fd_mark(L, FD_PH_FINALIZE, s);
  k_advance<T><<<1, 32, 0, s>>>(b);
  fd_mark(L, FD_PH_ADVANCE, s);
  return cudaGetLastError() == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
}

template <typename T>
int launch_cfl(const FDLaunch& L, const void* state, const FDArgs& a, cudaStream_t s) {
  Bufs<T> b = make_bufs<T>(L, const_cast<void*>(state), a);
  k_cfl<T><<<L.grid, kThreads, 0, s>>>(b);
  fd_mark(L, FD_PH_CFL, s);
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
