// Finite-volume MHD step as one persistent cooperative kernel.
//
// One launch runs whole time steps of the reference's FV path
// (astronomix/_finite_volume/_state_evolution/evolve_state.py:497-600):
//
//   dt      = C / sum_a max(|u_a| + c) / dx     _timestep_estimator.py:118-128
//   gas     = RK2(gas, dt/2)                    evolve_state.py:419-488
//   B, gas  = magnetic_update(B, gas, dt)       _magnetic_field_update.py:37-242
//   gas     = RK2(gas, dt/2)
//   t      += dt                                time_integration.py:737
//
// Each phase is a sweep over tiles; phases are separated by a bounded grid
// barrier (amx_common.cuh), so the global reductions of the step (the CFL
// maximum and the fixed-point residual of every magnetic iteration) never
// leave the device.  Every phase that writes the gas state also reduces the
// maxima of |u_a| + c over what it wrote: that is the Lax-Friedrichs alpha of
// the next stage and, after the last stage, the CFL estimate of the next
// step, so neither needs a sweep of its own.  A runtime `mode` runs a single seam instead of full
// steps, which is how the C-ABI exposes the reference's step-level functions.
//
// HBM layout: state[var][x][y][z] (C order, last axis contiguous), no ghost
// cells; boundary conditions are applied by index mapping at load time.
#pragma once

#include "amx_common.cuh"
#include "fv_physics.cuh"

namespace amx {

// Control block in device memory (one per plan).
struct FVControl {
  // zeroed before every launch (one memset up to `dt`)
  unsigned long long red[3][4];   // [slot][axis] maxima of |u_a| + c of a state a phase wrote
  unsigned long long spare[3][4];
  unsigned long long mag[3];      // [slot] fixed-point residual
  unsigned long long bar_count;   // grid-barrier arrivals of the current launch
  int abort_flag;
  int pad_b;
  // kept across launches
  double dt;                      // dt of the last step taken
  double t;                       // simulation time
  long long steps;                // steps taken
  int mag_iters;                  // fixed-point iterations of the last magnetic update
  int pad0;
  long long mag_iters_total;
  int status;
  int pad2;
  // device-driven seams (dt_dev): FV_MODE_DT sets dt and whether a step is
  // taken; the hydro seam records the maxima of |u_a| + c of its input state
  int active;
  int pad1;
  double seam_maxima[3];
};

enum FVScheme { FV_UNSPLIT = 0, FV_SPLIT = 1, FV_UNSPLIT_PP = 2 };

enum FVMode {
  FV_MODE_STEPS = 0,      // full time steps
  FV_MODE_CFL = 1,        // only the CFL dt (written to ctl->dt)
  FV_MODE_HYDRO_RK2 = 2,  // one RK2 update of the gas rows with dt_in * dt_scale
  FV_MODE_MAGNETIC = 3,   // one magnetic sub-step with dt_in
  FV_MODE_EVOLVE = 4,     // one _evolve_state_fv with dt_in (no CFL, no t update)
  FV_MODE_DT = 5,         // dt of the next step into ctl->dt, ctl->active = whether it is taken
};

template <typename T>
struct FVArgs {
  T* state;          // [nvars][ncells]
  T* p1;             // [nv_gas][ncells] RK stage buffer
  T* mag0;           // [6][ncells] magnetic iterate buffers
  T* mag1;
  FVControl* ctl;
  double* dt_hist;   // optional [max_hist] dt of every step (indexed by step number)
  int* it_hist;      // optional [max_hist] fixed-point iterations per step
  long long max_hist;
  int n;             // cells per axis
  long long ncells;
  AxisBC bc[3];
  int periodic_roll; // reference PERIODIC_ROLL boundary handling
  int limiter;
  int integrator;    // IMPLICIT_MIDPOINT / IMPLICIT_EULER
  int lm;            // HLLC-LM variant (riemann family HLLC)
  int am;            // family HLLC: 1 AM_HLLC, 2 HYBRID_HLLC (HLLC-LM where the right cell is compressed), 0 none
  int exact_end_time;
  int fixed_timestep;
  int mode;
  double dx;
  double inv_dx;     // 1 / dx (computed on the host)
  double gamma;
  double C_cfl;
  double t_end;
  double dt_fixed;   // t_end / num_timesteps (fixed mode)
  double dt_in;      // seam modes
  double dt_scale;   // seam modes
  int dt_dev;        // seam modes: dt from ctl->dt (times dt_scale), nothing done unless ctl->active
  double tol;        // fixed-point tolerance
  int max_iters;     // fixed-point cap (1000 in the reference)
  unsigned long long spin_limit;  // polls before a grid barrier gives up (AMX_ERR_TIMEOUT)
  int mhd;           // the state carries B (the magnetic split is active)
  int split;         // 1: dimensionally split MUSCL-Hancock sweeps instead of SSP-RK2
  int first_order;   // split: piecewise-constant interface states
  int use_dt_max;    // split: dt = min(dt, dt_max)
  double dt_max;
  T* p2;             // split: third sweep buffer (gas rows)
  long long max_steps;
  double t_pause;    // full-step mode stops before a step that starts at t >= t_pause
  // Tape mode (full steps): every intermediate state of every step is kept
  // in `tape` (see the tape layout at fv_run_kernel); null otherwise.
  T* tape;
  long long tape_cap;   // elements of `tape`
  long long* tape_off;  // [max_hist + 1] element offset of each step's start state
};

// per-item entry points, defined below
template <typename T, int DIM, int RS, int V> struct FVItems;
template <typename T, int DIM> struct MagItems;

// ---------------------------------------------------------------- tiles

template <typename T, int DIM> struct Tile;
template <typename T> struct Tile<T, 1> {
  static constexpr int T0 = 256, T1 = 1, T2 = 1;
};
template <> struct Tile<float, 2> {
  static constexpr int T0 = 16, T1 = 32, T2 = 1;
};
template <> struct Tile<double, 2> {
  static constexpr int T0 = 4, T1 = 64, T2 = 1;
};
template <> struct Tile<float, 3> {
  static constexpr int T0 = 4, T1 = 4, T2 = 32;
};
template <> struct Tile<double, 3> {
  static constexpr int T0 = 4, T1 = 4, T2 = 16;
};

// Alternative tile shapes the batched driver's autotuner chooses from
// (variant 0 is Tile<T, DIM>).
template <typename T, int DIM, int V> struct TileV : Tile<T, DIM> {};
template <typename T> struct TileV<T, 2, 1> {
  static constexpr int T0 = 4, T1 = 64, T2 = 1;
};
template <typename T> struct TileV<T, 2, 2> {
  static constexpr int T0 = 8, T1 = 64, T2 = 1;
};

constexpr int kFVThreads = 256;

// 3D FP32 magnetic evaluation streamed along axis 0 (mag_stream): a plane
// tile of kMS1 x kMS2 cells (axes 1, 2), one cell per thread, with a halo of
// one; a ring of four planes of six values (averaged B, E = B x v) per cell
// and two planes of the 13 inputs of each thread's own cell.
constexpr int kMS1 = 8, kMS2 = 32;
constexpr int kMSW2 = kMS2 + 2;
constexpr int kMSP = (kMS1 + 2) * kMSW2;
constexpr int kMSRing = 2 * kMS2 + 2 * kMS1;  // the plane's halo without its corners
constexpr int kMSRaw = 13;                    // B_k, v_k, B0, v0, rho
// planes ahead of the update whose rows mag_stream prefetches into L2 (0: none)
#ifndef AMX_MAG_PF
#define AMX_MAG_PF 4
#endif

static_assert(kMS1 * kMS2 == kFVThreads, "one cell of the plane tile per thread");
static_assert(kMSRing <= kFVThreads, "one halo entry per thread");

template <typename T, int DIM, int V = 0>
struct TileGeom {
  static constexpr int NV = DIM + 2;
  static constexpr int T0 = TileV<T, DIM, V>::T0, T1 = TileV<T, DIM, V>::T1, T2 = TileV<T, DIM, V>::T2;
  static constexpr int H0 = T0 + 4, H1 = (DIM >= 2) ? T1 + 4 : 1, H2 = (DIM >= 3) ? T2 + 4 : 1;
  static constexpr int HALO = H0 * H1 * H2;
  static constexpr int CELLS = T0 * T1 * T2;
  static constexpr int CPT = (CELLS + kFVThreads - 1) / kFVThreads;
  // faces of one axis and the cells (tile +- 1 along the axis) whose slopes they use
  static constexpr int F0 = (T0 + 1) * T1 * T2;
  static constexpr int F1 = (DIM >= 2) ? T0 * (T1 + 1) * T2 : 0;
  static constexpr int F2 = (DIM >= 3) ? T0 * T1 * (T2 + 1) : 0;
  static constexpr int FMAX = F0 > F1 ? (F0 > F2 ? F0 : F2) : (F1 > F2 ? F1 : F2);
  static constexpr int S0 = (T0 + 2) * T1 * T2;
  static constexpr int S1 = (DIM >= 2) ? T0 * (T1 + 2) * T2 : 0;
  static constexpr int S2 = (DIM >= 3) ? T0 * T1 * (T2 + 2) : 0;
  static constexpr int SMAX = S0 > S1 ? (S0 > S2 ? S0 : S2) : (S1 > S2 ? S1 : S2);
  // FUSED: all axes in one pass (slope and flux arrays side by side) instead
  // of one axis at a time; measured slower on GB300 for both 2D and 3D
  static constexpr bool FUSED = false;
  // 3D (HBM-bound) precomputes the limited slopes once per cell; up to 2D
  // (L2-resident, latency-bound) both faces evaluate them in registers
  static constexpr bool SLOPES = DIM == 3;
  static constexpr int SREG = SLOPES ? (FUSED ? S0 + S1 : SMAX) : 0;
  static constexpr int FREG = FUSED ? F0 + F1 : FMAX;
  // magnetic tile: halo 1, six values per cell (averaged B and E = B x v)
  static constexpr int M0 = T0 + 2, M1 = (DIM >= 2) ? T1 + 2 : 1, M2 = (DIM >= 3) ? T2 + 2 : 1;
  static constexpr int MHALO = M0 * M1 * M2;
  // FP32 3D: the halo tile starts two values into the buffer, so that the
  // interior of every halo row (the tile's own cells along axis 2) sits on a
  // 16-byte boundary for the 16-byte copies of hydro_tile
  static constexpr int SP_OFF = (DIM == 3 && V == 0 && sizeof(T) == 4) ? 2 : 0;
  static constexpr size_t HYDRO_SMEM = sizeof(T) * ((size_t)NV * (HALO + FREG + SREG) + SP_OFF);
  static constexpr size_t MAG_TILE_SMEM = sizeof(T) * (size_t)6 * MHALO;
  static constexpr size_t MAG_STREAM_SMEM =
      (DIM == 3 && V == 0 && sizeof(T) == 4) ? sizeof(T) * ((size_t)4 * 6 * kMSP + (size_t)2 * kMSRaw * kFVThreads) : 0;
  static constexpr size_t MAG_SMEM = MAG_TILE_SMEM > MAG_STREAM_SMEM ? MAG_TILE_SMEM : MAG_STREAM_SMEM;
  static constexpr size_t SMEM = HYDRO_SMEM > MAG_SMEM ? HYDRO_SMEM : MAG_SMEM;
  // VAN_ALBADA_PP: the limited differences of every axis for the tile and a
  // halo of 1, after the hydro arrays
  static constexpr int B0 = T0 + 2, B1 = (DIM >= 2) ? T1 + 2 : 1, B2 = (DIM >= 3) ? T2 + 2 : 1;
  static constexpr int BOX = B0 * B1 * B2;
  static constexpr size_t PP_SMEM = sizeof(T) * (size_t)DIM * NV * BOX;
  // split sweep along axis k: the tile with a halo of 2 along k, the faces
  // along k, and the interface states (left / right) of the cells beside them
  static constexpr int X0 = (T0 + 4) * T1 * T2 + (T0 + 1) * T1 * T2 + 2 * (T0 + 2) * T1 * T2;
  static constexpr int X1 = (DIM >= 2) ? T0 * ((T1 + 4) + (T1 + 1) + 2 * (T1 + 2)) * T2 : 0;
  static constexpr int X2 = (DIM >= 3) ? T0 * T1 * ((T2 + 4) + (T2 + 1) + 2 * (T2 + 2)) : 0;
  static constexpr int XMAX = X0 > X1 ? (X0 > X2 ? X0 : X2) : (X1 > X2 ? X1 : X2);
  static constexpr size_t SPLIT_SMEM0 = sizeof(T) * (size_t)NV * XMAX;
  static constexpr size_t SPLIT_SMEM = SPLIT_SMEM0 > SMEM ? SPLIT_SMEM0 : SMEM;
};

template <int DIM>
__host__ __device__ inline long long fv_num_tiles(int n, int T0, int T1, int T2) {
  long long t = (n + T0 - 1) / T0;
  if (DIM >= 2) t *= (n + T1 - 1) / T1;
  if (DIM >= 3) t *= (n + T2 - 1) / T2;
  return t;
}

template <int DIM>
__device__ __forceinline__ void tile_origin(long long tile, int n, int T0, int T1, int T2, int* o) {
  const int n1 = (DIM >= 2) ? (n + T1 - 1) / T1 : 1;
  const int n2 = (DIM >= 3) ? (n + T2 - 1) / T2 : 1;
  const int t2 = (int)(tile % n2);
  const int t1 = (int)((tile / n2) % n1);
  const int t0 = (int)(tile / ((long long)n2 * n1));
  o[0] = t0 * T0;
  o[1] = t1 * T1;
  o[2] = t2 * T2;
}

template <int DIM>
__device__ __forceinline__ long long cell_index(int i0, int i1, int i2, int n) {
  if (DIM == 1) return i0;
  if (DIM == 2) return (long long)i0 * n + i1;
  return ((long long)i0 * n + i1) * n + i2;
}

// Maps a logical (possibly out-of-domain, clamped to [-2, n+1]) index onto
// the stored grid.  The boundary settings are copied into registers: FVArgs
// is read through a reference, so its fields would be reloaded after every
// store.
template <int DIM>
struct AxisMap {
  int n;
  bool roll;
  bool reflective;  // some wall of the first DIM axes mirrors (and flips a velocity)
  AxisBC bc[3];
  template <typename T>
  __device__ __forceinline__ explicit AxisMap(const FVArgs<T>& a) : n(a.n), roll(a.periodic_roll != 0) {
    reflective = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      bc[k] = a.bc[k];
      if (k < DIM && (bc[k].lo == AMX_BC_REFLECTIVE || bc[k].hi == AMX_BC_REFLECTIVE)) reflective = true;
    }
    if (roll) reflective = false;
  }
  __device__ __forceinline__ int operator()(int k, int g, bool* flip) const {
    if (g < -2) g = -2;
    if (g > n + 1) g = n + 1;
    if (roll) return wrap(g, n);
    return map_index(g, n, bc[k], DIM == 1, flip);
  }
};

// ------------------------------------------------------------ reductions

// Folds per-thread maxima of |u_a| + c into `slot` (block max + atomicMax).
// The maxima are tracked in the state's precision (a maximum is exact in any
// precision) and widened to FP64 once per block: GB300's FP64 rate is a small
// fraction of its FP32 rate.
template <int DIM, typename T>
__device__ __forceinline__ void fold_maxima(const T* m, unsigned long long* slot, double* red) {
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    const double r = block_max<double>((double)m[k], red);
    if (threadIdx.x == 0) atomic_max_nonneg(&slot[k], r);
  }
}

template <typename T, int DIM>
__device__ __forceinline__ void track_maxima(const T* q, T gamma, T* m) {
  const T cs = sound_speed(q[0], q[DIM + 1], gamma);
#pragma unroll
  for (int k = 0; k < DIM; ++k) m[k] = nanmax(m[k], Num<T>::abs_(q[1 + k]) + cs);
}

// Per-axis maxima of |u_a| + c over all cells of the state (the reference's
// ghost cells are copies of interior cells and add nothing to the maximum).
template <typename T, int DIM>
__device__ __noinline__ void phase_cfl(const FVArgs<T>& a, const T* st, unsigned long long* slot, double* red) {
  const T gamma = T(a.gamma);
  T m[3] = {T(0), T(0), T(0)};
  const long long nc = a.ncells;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (long long)gridDim.x * blockDim.x) {
    T q[DIM + 2];
#pragma unroll
    for (int v = 0; v < DIM + 2; ++v) q[v] = st[v * nc + c];
    track_maxima<T, DIM>(q, gamma, m);
  }
  fold_maxima<DIM>(m, slot, red);
}

// ------------------------------------------------------------ hydro stage

// The VAN_ALBADA_PP rescaling of one cell's differences d[k][v] (limited
// gradient x dx/2 along axis k) for positivity (reconstruction.py:167-362):
// the density and pressure differences of axis k by alpha_k, kappa_k, the
// velocity differences by one beta per cell.  C[k] = a_k / sum(a) from the
// global maxima a_k of |u_k| + c; q = 2 / C_cfl with MHD, 1 / C_cfl
// without.  A1 pairs C, alpha and the density difference of axis j with
// velocity component j, as the reference's array broadcasting does.
template <typename T, int DIM>
__device__ __forceinline__ void pp_limit(T (*d)[DIM + 2], T rho, T p, const T* C, T q, T gamma) {
  constexpr int P = DIM + 1;
  const T eps = T(1e-14);
  T alpha[DIM], kappa[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    const T dr = d[k][0], dp = d[k][P];
    alpha[k] = Num<T>::abs_(dr) > eps ? jmin(rho / (Num<T>::abs_(dr) * (T(1) + eps)), T(1)) : T(1);
    kappa[k] = Num<T>::abs_(dp) > eps ? jmin(p / (Num<T>::abs_(dp) * (T(1) + eps)), T(1)) : T(1);
  }
  T A1 = T(0), A2 = T(0), vsum = T(0);
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    const T X = C[j] * alpha[j] * d[j][0];
    T S = X * d[0][1 + j];
#pragma unroll
    for (int k = 1; k < DIM; ++k) S = S + X * d[k][1 + j];
    A1 = (j == 0) ? S * S : A1 + S * S;
  }
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    T sq = d[k][1] * d[k][1];
#pragma unroll
    for (int j = 1; j < DIM; ++j) sq = sq + d[k][1 + j] * d[k][1 + j];
    A2 = (k == 0) ? C[k] * sq : A2 + C[k] * sq;
    vsum = (k == 0) ? sq : vsum + sq;
  }
  const bool moving = vsum > eps;
  if (!moving) { A1 = eps; A2 = eps; }
  const T qm2 = q - T(2);
  const T beta = moving ? jmin(Num<T>::sqrt_((qm2 * qm2 * rho * p) /
                                             ((gamma - T(1)) * (T(2) * A1 + qm2 * (rho * rho) * A2))), T(1))
                        : T(1);
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    d[k][0] = d[k][0] * alpha[k];
    d[k][P] = d[k][P] * kappa[k];
#pragma unroll
    for (int j = 0; j < DIM; ++j) d[k][1 + j] = d[k][1 + j] * beta;
  }
}

// VAN_ALBADA_PP pre-pass of a hydro tile: the rescaled differences of every
// axis for the tile and a halo of 1 from the staged primitives sP into sPP
// ([DIM][NV][BOX]).  Out of line, so that the registers it needs do not
// weigh on the hydro stage of the other limiters.
template <typename T, int DIM, int V>
__device__ __noinline__ void pp_prepass(const FVArgs<T>& a, const T* sP, T* sPP, const T* ppC) {
  using G = TileGeom<T, DIM, V>;
  constexpr int NV = G::NV;
  const T gamma = T(a.gamma);
  const T dxT = T(a.dx);
  const int limiter = a.limiter;
  const T q = T(a.mhd ? 2 : 1) / T(a.C_cfl);  // the hydro half steps of the MHD split count as C_cfl / 2
  for (int e = threadIdx.x; e < G::BOX; e += blockDim.x) {
    const int b2 = e % G::B2, b1 = (e / G::B2) % G::B1, b0 = e / (G::B2 * G::B1);
    const int hh = ((b0 + 1) * G::H1 + (DIM >= 2 ? b1 + 1 : 0)) * G::H2 + (DIM >= 3 ? b2 + 1 : 0);
    T d[DIM][DIM + 2];
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const int stride = (k == 0) ? G::H1 * G::H2 : ((k == 1) ? G::H2 : 1);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const T* s = sP + v * G::HALO + hh;
        d[k][v] = limited((s[0] - s[-stride]) / dxT, (s[stride] - s[0]) / dxT, limiter, dxT) * dxT / T(2);
      }
    }
    pp_limit<T, DIM>(d, sP[hh], sP[(NV - 1) * G::HALO + hh], ppC, q, gamma);
#pragma unroll
    for (int k = 0; k < DIM; ++k)
#pragma unroll
      for (int v = 0; v < NV; ++v) sPP[(k * NV + v) * G::BOX + e] = d[k][v];
  }
}

// One _evolve_gas_state_unsplit_inner (evolve_state.py:339-414):
//   U = cons(P_in); for each axis: U += (1/dx) (F[i-1/2] - F[i+1/2]) dt;
//   P_out = prim(U)
// and, when `P0` is given, the RK2 combination of evolve_state.py:456-469:
//   P_out = prim(0.5 (cons(P0) + cons(prim(U)))).
// `alpha` holds the Lax-Friedrichs alpha per axis (unused otherwise).  The
// limited slope of every cell (reconstruction.py:399-431) is computed once
// per axis into shared memory and read by both of its faces.  The maxima of
// |u_a| + c of P_out are folded into `out_slot`.
template <typename T, int DIM, int RS, int V = 0, bool PP = false>
__device__ __forceinline__ void hydro_tile(const FVArgs<T>& a, const int* o, const T* __restrict__ Pin, T* Pout,
                                           const T* P0, T dt, const T* alpha, T* smem, T* m, bool track,
                                           const T* ppC = nullptr) {
  using G = TileGeom<T, DIM, V>;
  constexpr int NV = G::NV;
  const int n = a.n;
  const long long nc = a.ncells;
  const T gamma = T(a.gamma);
  const T dxT = T(a.dx);
  const T inv_dx = T(a.inv_dx);
  const int limiter = a.limiter;
  const bool lm = a.lm != 0;
  const AxisMap<DIM> amap(a);
  T* sP = smem + G::SP_OFF;            // [NV][HALO]
  T* sF = sP + NV * G::HALO;           // [NV][FMAX]
  T* sD = sF + NV * G::FMAX;           // [NV][SMAX] slopes (already * dx / 2)

  // ---- load the halo'd tile of primitives (boundary-mapped)
  if constexpr (DIM == 3) {
    // 3D (4.5 halo cells per tile cell): every thread issues all of its
    // copies (cp.async) before waiting for any; a reflective wall's sign
    // flips are applied afterwards.  FP32, when the grid and the input
    // allow it: the tile's own cells of each halo row (axis 2, in range and
    // 16-byte aligned) go as 16-byte copies, four values each, and the two
    // halo cells at either end as mapped single values: the index arithmetic
    // is done per row and per copy of four rather than per value.
    bool rows = false;
    if constexpr (G::SP_OFF == 2) {
      static_assert(G::T2 % 4 == 0 && G::H2 == G::T2 + 4 && G::HALO % 4 == 0 && G::H2 % 4 == 0,
                    "16-byte row copies: the row interior starts two values in");
      rows = (n % 4 == 0) && (o[2] + G::T2 <= n) && ((reinterpret_cast<unsigned long long>(Pin) & 15ull) == 0);
    }
    if (rows) {
      constexpr int Q = G::T2 / 4;      // 16-byte copies per row
      constexpr int SLOTS = Q + 4;      // and the four mapped end cells
      constexpr int NROWS = G::H0 * G::H1;
      for (int it = threadIdx.x; it < NROWS * SLOTS; it += blockDim.x) {
        const int row = it / SLOTS, sl = it % SLOTS;
        const int h0 = row / G::H1, h1 = row % G::H1;
        bool f = false;
        const long long base = ((long long)amap(0, o[0] + h0 - 2, &f) * n + amap(1, o[1] + h1 - 2, &f)) * n;
        if (sl < Q) {
          const int j = 2 + 4 * sl;  // halo column of the copy's first value
          const long long c = base + o[2] + 4 * sl;
#pragma unroll
          for (int v = 0; v < NV; ++v) cp_async_16(sP + v * G::HALO + row * G::H2 + j, Pin + v * nc + c);
        } else {
          const int k = sl - Q;                     // 0, 1: left of the tile; 2, 3: right
          const int j = (k < 2) ? k : G::T2 + k;    // halo columns 0, 1, T2 + 2, T2 + 3
          const long long c = base + amap(2, o[2] + j - 2, &f);
#pragma unroll
          for (int v = 0; v < NV; ++v) cp_async_elem(sP + v * G::HALO + row * G::H2 + j, Pin + v * nc + c);
        }
      }
    } else {
      for (int e = threadIdx.x; e < G::HALO; e += blockDim.x) {
        const int h2 = e % G::H2;
        const int h1 = (e / G::H2) % G::H1;
        const int h0 = e / (G::H2 * G::H1);
        bool f = false;
        const long long c =
            cell_index<DIM>(amap(0, o[0] + h0 - 2, &f), amap(1, o[1] + h1 - 2, &f), amap(2, o[2] + h2 - 2, &f), n);
#pragma unroll
        for (int v = 0; v < NV; ++v) cp_async_elem(sP + v * G::HALO + e, Pin + v * nc + c);
      }
    }
    cp_async_commit();
    cp_async_wait_all();
    if (amap.reflective) {
      for (int e = threadIdx.x; e < G::HALO; e += blockDim.x) {
        const int h2 = e % G::H2;
        const int h1 = (e / G::H2) % G::H1;
        const int h0 = e / (G::H2 * G::H1);
        bool f0 = false, f1 = false, f2 = false;
        amap(0, o[0] + h0 - 2, &f0);
        amap(1, o[1] + h1 - 2, &f1);
        amap(2, o[2] + h2 - 2, &f2);
        if (f0) sP[1 * G::HALO + e] = -sP[1 * G::HALO + e];
        if (f1) sP[2 * G::HALO + e] = -sP[2 * G::HALO + e];
        if (f2) sP[3 * G::HALO + e] = -sP[3 * G::HALO + e];
      }
    }
  } else {
    for (int e = threadIdx.x; e < G::HALO; e += blockDim.x) {
      const int h2 = e % G::H2;
      const int h1 = (e / G::H2) % G::H1;
      const int h0 = e / (G::H2 * G::H1);
      bool f0 = false, f1 = false, f2 = false;
      const int i0 = amap(0, o[0] + h0 - 2, &f0);
      const int i1 = (DIM >= 2) ? amap(1, o[1] + h1 - 2, &f1) : 0;
      const int i2 = (DIM >= 3) ? amap(2, o[2] + h2 - 2, &f2) : 0;
      const long long c = cell_index<DIM>(i0, i1, i2, n);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        T val = Pin[v * nc + c];
        if ((v == 1 && f0) || (v == 2 && f1) || (v == 3 && f2)) val = -val;
        sP[v * G::HALO + e] = val;
      }
    }
  }
  __syncthreads();

  // ---- VAN_ALBADA_PP: the rescaled differences of every axis for the tile
  // and a halo of 1, before any face needs them (reconstruction.py:134-394)
  T* sPP = sP + NV * (G::HALO + G::FREG + G::SREG);  // [DIM][NV][BOX]
  if (PP) {
    pp_prepass<T, DIM, V>(a, sP, sPP, ppC);
    __syncthreads();
  }

  // ---- per-thread cells: conserved state from the (mapped) primitives
  T U[G::CPT][NV];
#pragma unroll
  for (int j = 0; j < G::CPT; ++j) {
    const int cl = threadIdx.x + j * kFVThreads;
    if (cl < G::CELLS) {
      const int c2 = cl % G::T2, c1 = (cl / G::T2) % G::T1, c0 = cl / (G::T2 * G::T1);
      const int h = ((c0 + 2) * G::H1 + (DIM >= 2 ? c1 + 2 : 0)) * G::H2 + (DIM >= 3 ? c2 + 2 : 0);
      T q[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) q[v] = sP[v * G::HALO + h];
      prim_to_cons<T, DIM>(q, U[j], gamma);
    }
  }

  // ---- axes in the reference order x, y, z.  Fused (DIM <= 2): slopes of
  // all axes, one barrier, fluxes of all axes, one barrier, then every cell
  // adds its x and then its y flux differences.  3D: one axis at a time.
  constexpr int NPASS = G::FUSED ? 1 : DIM;
#pragma unroll
  for (int pass = 0; pass < NPASS; ++pass) {
    const int k_lo = G::FUSED ? 0 : pass, k_hi = G::FUSED ? DIM : pass + 1;
    for (int k = k_lo; k < ((G::SLOPES && !PP) ? k_hi : k_lo); ++k) {
      const int stride = (k == 0) ? G::H1 * G::H2 : ((k == 1) ? G::H2 : 1);
      const int D0 = G::T0 + 2 * (k == 0), D1 = (DIM >= 2) ? G::T1 + 2 * (k == 1) : 1,
                D2 = (DIM >= 3) ? G::T2 + 2 * (k == 2) : 1;
      const int ns = D0 * D1 * D2;
      T* sDk = sD + ((G::FUSED && k == 1) ? NV * G::S0 : 0);
      const int sdim = G::FUSED ? (k == 0 ? G::S0 : G::S1) : G::SMAX;
      for (int e = threadIdx.x; e < ns; e += blockDim.x) {
        const int d2 = e % D2, d1 = (e / D2) % D1, d0 = e / (D2 * D1);
        const int h = ((d0 + 2 - (k == 0)) * G::H1 + (DIM >= 2 ? d1 + 2 - (k == 1) : 0)) * G::H2 +
                      (DIM >= 3 ? d2 + 2 - (k == 2) : 0);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const T* s = sP + v * G::HALO + h;
          const T qm = s[-stride], q0 = s[0], qp = s[stride];
          sDk[v * sdim + e] = half_slope(qm, q0, qp, limiter, dxT);
        }
      }
    }
    if (G::SLOPES && !PP) __syncthreads();
    for (int k = k_lo; k < k_hi; ++k) {
      const int stride = (k == 0) ? G::H1 * G::H2 : ((k == 1) ? G::H2 : 1);
      const int D1 = (DIM >= 2) ? G::T1 + 2 * (k == 1) : 1, D2 = (DIM >= 3) ? G::T2 + 2 * (k == 2) : 1;
      const T* sDk = sD + ((G::FUSED && k == 1) ? NV * G::S0 : 0);
      const int sdim = G::FUSED ? (k == 0 ? G::S0 : G::S1) : G::SMAX;
      T* sFk = sF + ((G::FUSED && k == 1) ? NV * G::F0 : 0);
      const int fdim = G::FUSED ? (k == 0 ? G::F0 : G::F1) : G::FMAX;
      const int E0 = G::T0 + (k == 0), E1 = (DIM >= 2) ? G::T1 + (k == 1) : 1,
                E2 = (DIM >= 3) ? G::T2 + (k == 2) : 1;
      const int nf = E0 * E1 * E2;
      const int dstride = (k == 0) ? D1 * D2 : ((k == 1) ? D2 : 1);
      for (int f = threadIdx.x; f < nf; f += blockDim.x) {
        const int f2 = f % E2, f1 = (f / E2) % E1, f0 = f / (E2 * E1);
        // halo index of the cell right of the face (local cell c = face index)
        const int h = ((f0 + 2) * G::H1 + (DIM >= 2 ? f1 + 2 : 0)) * G::H2 + (DIM >= 3 ? f2 + 2 : 0);
        // slope index of that cell (slope arrays start one cell before the tile along k)
        const int ds = (f0 + (k == 0)) * D1 * D2 + (DIM >= 2 ? (f1 + (k == 1)) * D2 : 0) +
                       (DIM >= 3 ? f2 + (k == 2) : 0);
        T qL[NV], qR[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const T* s = sP + v * G::HALO + h;
          if (PP) {
            // box index of the cell right of the face, and of its left neighbour along k
            const int br = ((f0 + 1) * G::B1 + (DIM >= 2 ? f1 + 1 : 0)) * G::B2 + (DIM >= 3 ? f2 + 1 : 0);
            const int bl = br - ((k == 0) ? G::B1 * G::B2 : ((k == 1) ? G::B2 : 1));
            const T* dd = sPP + (k * NV + v) * G::BOX;
            qL[v] = s[-stride] + dd[bl];
            qR[v] = s[0] - dd[br];
          } else if (G::SLOPES) {
            const T* d = sDk + v * sdim + ds;
            qL[v] = s[-stride] + d[-dstride];
            qR[v] = s[0] - d[0];
          } else {
            const T qm2 = s[-2 * stride], qm1 = s[-stride], q0 = s[0], qp1 = s[stride];
            qL[v] = qm1 + half_slope(qm2, qm1, q0, limiter, dxT);
            qR[v] = q0 - half_slope(qm1, q0, qp1, limiter, dxT);
          }
        }
        T F[NV];
        bool lmf = lm;
        if constexpr (RS == RS_AM) {
          // hll.py:268-326: the switch of the cell right of the face (the
          // reference's flux index i is the face i - 1/2)
          const int strides[3] = {G::H1 * G::H2, G::H2, 1};
          lmf = am_compressed<T, DIM>(sP + h, G::HALO, strides, gamma, dxT);
        }
        riemann<T, DIM, RS>(qL, qR, k + 1, gamma, alpha ? alpha[k] : T(0), lmf, F, a.am == 1);
#pragma unroll
        for (int v = 0; v < NV; ++v) sFk[v * fdim + f] = F[v];
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < G::CPT; ++j) {
      const int cl = threadIdx.x + j * kFVThreads;
      if (cl < G::CELLS) {
        const int c2 = cl % G::T2, c1 = (cl / G::T2) % G::T1, c0 = cl / (G::T2 * G::T1);
        for (int k = k_lo; k < k_hi; ++k) {
          const T* sFk = sF + ((G::FUSED && k == 1) ? NV * G::F0 : 0);
          const int fdim = G::FUSED ? (k == 0 ? G::F0 : G::F1) : G::FMAX;
          const int E1 = (DIM >= 2) ? G::T1 + (k == 1) : 1, E2 = (DIM >= 3) ? G::T2 + (k == 2) : 1;
          const int fl = (c0 * E1 + c1) * E2 + c2;  // face i-1/2 of the cell
          const int fr = fl + ((k == 0) ? E1 * E2 : ((k == 1) ? E2 : 1));
#pragma unroll
          for (int v = 0; v < NV; ++v)
            U[j][v] = U[j][v] + inv_dx * (sFk[v * fdim + fl] - sFk[v * fdim + fr]) * dt;
        }
      }
    }
    if (!G::FUSED) __syncthreads();
  }

  // ---- back to primitives (+ RK2 combination) and store
#pragma unroll
  for (int j = 0; j < G::CPT; ++j) {
    const int cl = threadIdx.x + j * kFVThreads;
    if (cl < G::CELLS) {
      const int c2 = cl % G::T2, c1 = (cl / G::T2) % G::T1, c0 = cl / (G::T2 * G::T1);
      const int g0 = o[0] + c0, g1 = o[1] + c1, g2 = o[2] + c2;
      if (g0 < n && (DIM < 2 || g1 < n) && (DIM < 3 || g2 < n)) {
        const long long c = cell_index<DIM>(g0, g1, g2, n);
        T q[NV];
        cons_to_prim<T, DIM>(U[j], q, gamma);
        if (P0) {
          T U2[NV], q0[NV], U0[NV];
          prim_to_cons<T, DIM>(q, U2, gamma);
#pragma unroll
          for (int v = 0; v < NV; ++v) q0[v] = P0[v * nc + c];
          prim_to_cons<T, DIM>(q0, U0, gamma);
#pragma unroll
          for (int v = 0; v < NV; ++v) U2[v] = T(0.5) * (U0[v] + U2[v]);
          cons_to_prim<T, DIM>(U2, q, gamma);
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) Pout[v * nc + c] = q[v];
        if (track) track_maxima<T, DIM>(q, gamma, m);
      }
    }
  }
  if (G::FUSED) __syncthreads();  // the flux arrays are read above; the next tile overwrites them
}

template <typename T, int DIM, int RS, bool PP = false>
__device__ __noinline__ void phase_hydro_stage(const FVArgs<T>& a, const T* __restrict__ Pin, T* Pout,
                                               const T* P0, T dt, const T* alpha, T* smem,
                                               unsigned long long* out_slot, double* red, const T* ppC = nullptr) {
  using G = TileGeom<T, DIM>;
  const long long ntiles = fv_num_tiles<DIM>(a.n, G::T0, G::T1, G::T2);
  T m[3] = {T(0), T(0), T(0)};
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int o[3];
    tile_origin<DIM>(tile, a.n, G::T0, G::T1, G::T2, o);
    FVItems<T, DIM, RS, 0>::template hydro<PP>(a, o, Pin, Pout, P0, dt, alpha, smem, m, out_slot != nullptr, ppC);
  }
  if (out_slot) fold_maxima<DIM>(m, out_slot, red);
}

// ------------------------------------------------------------ split sweep

// MUSCL-Hancock interface state of cell X (reconstruction.py:40-129,
// Cartesian): the limited gradient g along the sweep axis (1-based velocity
// index d), the half-step predictor q - dt/2 A_W g with the reference's A_W
// (u on the diagonal, A[rho][d] = rho, A[p][1] = rho c^2 -- velocity
// column 1 whatever the axis, as the reference sets it --, A[d][p] = 1/rho;
// the products summed in increasing column order), then
// predictor -/+ (dx/2) g at the cell's left / right interface.
template <typename T, int DIM>
__device__ __forceinline__ void muscl_states(const T* qm, const T* q0, const T* qp, int d, T gamma, T dt, T dxT,
                                             int limiter, T* left, T* right) {
  constexpr int NV = DIM + 2, P = DIM + 1;
  T g[NV];
  if constexpr (sizeof(T) == 4) {
    if (limiter == 0) {
      // FP32 MINMOD: the minmod of the differences, divided by dx once
      const T rdx = T(1) / dxT;
#pragma unroll
      for (int v = 0; v < NV; ++v) g[v] = minmod_cases(q0[v] - qm[v], qp[v] - q0[v]) * rdx;
    } else {
#pragma unroll
      for (int v = 0; v < NV; ++v) g[v] = limited((q0[v] - qm[v]) / dxT, (qp[v] - q0[v]) / dxT, limiter, dxT);
    }
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) g[v] = limited((q0[v] - qm[v]) / dxT, (qp[v] - q0[v]) / dxT, limiter, dxT);
  }
  const T rho = q0[0], u = q0[d];
  const T c = sound_speed(rho, q0[P], gamma);
  const T half = dt / T(2), dist = dxT / T(2);
#pragma unroll
  for (int b = 0; b < NV; ++b) {
    T proj;
    if (b == 0) proj = u * g[0] + rho * g[d];
    else if (b == d) proj = u * g[d] + (T(1) / rho) * g[P];
    else if (b == P) proj = (rho * (c * c)) * g[1] + u * g[P];
    else proj = u * g[b];
    const T pred = q0[b] - half * proj;
    left[b] = pred - dist * g[b];
    right[b] = pred + dist * g[b];
  }
}

// One split sweep of a tile along axis k (evolve_state.py:52-160):
// interface states (MUSCL-Hancock, or piecewise constant with
// first_order), Riemann fluxes along k, U += (1/dx)(F[i-1/2] - F[i+1/2]) dt.
// The tile carries a halo of 2 along k only.  The MUSCL-Hancock states of
// every cell beside a face are computed once into shared memory (both faces
// of a cell read them) before the Riemann pass.
template <typename T, int DIM, int RS, int K>
__device__ __forceinline__ void sweep_tile(const FVArgs<T>& a, const int* o, const T* __restrict__ Pin, T* Pout,
                                           T dt, const T* alpha, T* smem, T* m, bool track) {
  using G = TileGeom<T, DIM>;
  // the axis is a compile-time constant: the tile extents below are then
  // constants and the index arithmetic of every loop avoids integer division
  constexpr int k = K;
  constexpr int NV = G::NV;
  const int n = a.n;
  const long long nc = a.ncells;
  const T gamma = T(a.gamma);
  const T dxT = T(a.dx);
  const T inv_dx = T(a.inv_dx);
  const int limiter = a.limiter;
  const bool lm = a.lm != 0;
  const bool first_order = a.first_order != 0;
  const AxisMap<DIM> amap(a);
  constexpr int E0 = G::T0 + 4 * (k == 0), E1 = (DIM >= 2) ? G::T1 + 4 * (k == 1) : 1,
                E2 = (DIM >= 3) ? G::T2 + 4 * (k == 2) : 1;
  constexpr int HL = E0 * E1 * E2;
  constexpr int F0 = G::T0 + (k == 0), F1 = (DIM >= 2) ? G::T1 + (k == 1) : 1,
                F2 = (DIM >= 3) ? G::T2 + (k == 2) : 1;
  constexpr int NF = F0 * F1 * F2;
  constexpr int stride = (k == 0) ? E1 * E2 : ((k == 1) ? E2 : 1);
  // the cells beside a face along k: halo index 1 .. E_k - 2 along k
  constexpr int S0 = G::T0 + 2 * (k == 0), S1 = (DIM >= 2) ? G::T1 + 2 * (k == 1) : 1,
                S2 = (DIM >= 3) ? G::T2 + 2 * (k == 2) : 1;
  constexpr int NS = S0 * S1 * S2;
  constexpr int sstride = (k == 0) ? S1 * S2 : ((k == 1) ? S2 : 1);
  T* sP = smem;            // [NV][HL]
  T* sF = smem + NV * HL;  // [NV][NF]
  T* sLo = sF + NV * NF;   // [NV][NS] left-face state of each cell
  T* sHi = sLo + NV * NS;  // [NV][NS] right-face state
  for (int e = threadIdx.x; e < HL; e += blockDim.x) {
    const int e2 = e % E2, e1 = (e / E2) % E1, e0 = e / (E2 * E1);
    bool f0 = false, f1 = false, f2 = false;
    const int i0 = amap(0, o[0] + e0 - 2 * (k == 0), &f0);
    const int i1 = (DIM >= 2) ? amap(1, o[1] + e1 - 2 * (k == 1), &f1) : 0;
    const int i2 = (DIM >= 3) ? amap(2, o[2] + e2 - 2 * (k == 2), &f2) : 0;
    const long long c = cell_index<DIM>(i0, i1, i2, n);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      T val = Pin[v * nc + c];
      if ((v == 1 && f0) || (v == 2 && f1) || (v == 3 && f2)) val = -val;
      sP[v * HL + e] = val;
    }
  }
  __syncthreads();
  if (!first_order) {
    // MUSCL-Hancock states of the cells beside the faces, once per cell
    for (int e = threadIdx.x; e < NS; e += blockDim.x) {
      const int s2 = e % S2, s1 = (e / S2) % S1, s0 = e / (S2 * S1);
      const int h = ((s0 + (k == 0)) * E1 + (DIM >= 2 ? s1 + (k == 1) : 0)) * E2 + (DIM >= 3 ? s2 + (k == 2) : 0);
      T qm[NV], q0[NV], qp[NV], lo[NV], hi[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        qm[v] = sP[v * HL + h - stride];
        q0[v] = sP[v * HL + h];
        qp[v] = sP[v * HL + h + stride];
      }
      muscl_states<T, DIM>(qm, q0, qp, k + 1, gamma, dt, dxT, limiter, lo, hi);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        sLo[v * NS + e] = lo[v];
        sHi[v * NS + e] = hi[v];
      }
    }
    __syncthreads();
  }
  for (int f = threadIdx.x; f < NF; f += blockDim.x) {
    const int f2 = f % F2, f1 = (f / F2) % F1, f0 = f / (F2 * F1);
    T qL[NV], qR[NV];
    if (first_order) {
      // halo index of the cell right of the face
      const int hr = ((f0 + 2 * (k == 0)) * E1 + (DIM >= 2 ? f1 + 2 * (k == 1) : 0)) * E2 +
                     (DIM >= 3 ? f2 + 2 * (k == 2) : 0);
      const int hl = hr - stride;
#pragma unroll
      for (int v = 0; v < NV; ++v) { qL[v] = sP[v * HL + hl]; qR[v] = sP[v * HL + hr]; }
    } else {
      // the left cell of the face has index f_k along k in the state box, the right one f_k + 1
      const int sl = (f0 * S1 + (DIM >= 2 ? f1 : 0)) * S2 + (DIM >= 3 ? f2 : 0);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        qL[v] = sHi[v * NS + sl];            // right extrapolation of the left cell
        qR[v] = sLo[v * NS + sl + sstride];  // left extrapolation of the right cell
      }
    }
    T F[NV];
    bool lmf = lm;
    if constexpr (RS == RS_AM) {
      // hll.py:268-326 with the sweep's input state (evolve_state.py:80-88):
      // the compression switch of the cell right of the face, as
      // am_compressed forms it.  Its neighbours along the sweep axis are
      // staged; along the other axes they come from global memory through
      // the boundary map (a reflective wall negates its axis's velocity).
      const int hr = ((f0 + 2 * (k == 0)) * E1 + (DIM >= 2 ? f1 + 2 * (k == 1) : 0)) * E2 +
                     (DIM >= 3 ? f2 + 2 * (k == 2) : 0);
      const int fc[3] = {f0, f1, f2};
      int gi[3] = {0, 0, 0};
      bool fl_ = false;
#pragma unroll
      for (int b = 0; b < DIM; ++b) gi[b] = amap(b, o[b] + fc[b], &fl_);
      T div = T(0);
#pragma unroll
      for (int ax = 0; ax < DIM; ++ax) {
        T vp, vm;
        if (ax == k) {
          vp = sP[(1 + ax) * HL + hr + stride];
          vm = sP[(1 + ax) * HL + hr - stride];
        } else {
          bool fp = false, fm = false;
          int ip[3] = {gi[0], gi[1], gi[2]}, im[3] = {gi[0], gi[1], gi[2]};
          ip[ax] = amap(ax, o[ax] + fc[ax] + 1, &fp);
          im[ax] = amap(ax, o[ax] + fc[ax] - 1, &fm);
          vp = Pin[(1 + ax) * nc + cell_index<DIM>(ip[0], ip[1], ip[2], n)];
          vm = Pin[(1 + ax) * nc + cell_index<DIM>(im[0], im[1], im[2], n)];
          if (fp) vp = -vp;
          if (fm) vm = -vm;
        }
        div = div + (vp - vm) / (T(2) * dxT);
      }
      const T c = sound_speed(sP[hr], sP[(DIM + 1) * HL + hr], gamma);
      lmf = div < T(-0.05) * c / dxT;
    }
    riemann<T, DIM, RS>(qL, qR, k + 1, gamma, alpha ? alpha[k] : T(0), lmf, F, a.am == 1);
#pragma unroll
    for (int v = 0; v < NV; ++v) sF[v * NF + f] = F[v];
  }
  __syncthreads();
  constexpr int fstride = (k == 0) ? F1 * F2 : ((k == 1) ? F2 : 1);
  for (int cl = threadIdx.x; cl < G::CELLS; cl += blockDim.x) {
    const int c2 = cl % G::T2, c1 = (cl / G::T2) % G::T1, c0 = cl / (G::T2 * G::T1);
    const int g0 = o[0] + c0, g1 = o[1] + c1, g2 = o[2] + c2;
    if (!(g0 < n && (DIM < 2 || g1 < n) && (DIM < 3 || g2 < n))) continue;
    const int h = ((c0 + 2 * (k == 0)) * E1 + (DIM >= 2 ? c1 + 2 * (k == 1) : 0)) * E2 +
                  (DIM >= 3 ? c2 + 2 * (k == 2) : 0);
    const int fl = (c0 * F1 + (DIM >= 2 ? c1 : 0)) * F2 + (DIM >= 3 ? c2 : 0);  // face i-1/2
    const int fr = fl + fstride;
    T q[NV], U[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) q[v] = sP[v * HL + h];
    prim_to_cons<T, DIM>(q, U, gamma);
#pragma unroll
    for (int v = 0; v < NV; ++v) U[v] = U[v] + inv_dx * (sF[v * NF + fl] - sF[v * NF + fr]) * dt;
    cons_to_prim<T, DIM>(U, q, gamma);
    const long long c = cell_index<DIM>(g0, g1, g2, n);
#pragma unroll
    for (int v = 0; v < NV; ++v) Pout[v * nc + c] = q[v];
    if (track) track_maxima<T, DIM>(q, gamma, m);
  }
  __syncthreads();  // the next tile overwrites the shared arrays
}

template <typename T, int DIM, int RS>
__device__ __noinline__ void phase_sweep(const FVArgs<T>& a, int k, const T* __restrict__ Pin, T* Pout, T dt,
                                         const T* alpha, T* smem, unsigned long long* out_slot, double* red) {
  using G = TileGeom<T, DIM>;
  const long long ntiles = fv_num_tiles<DIM>(a.n, G::T0, G::T1, G::T2);
  T m[3] = {T(0), T(0), T(0)};
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int o[3];
    tile_origin<DIM>(tile, a.n, G::T0, G::T1, G::T2, o);
    if (k == 0)
      sweep_tile<T, DIM, RS, 0>(a, o, Pin, Pout, dt, alpha, smem, m, out_slot != nullptr);
    else if (DIM >= 2 && k == 1)
      sweep_tile<T, DIM, RS, (DIM >= 2 ? 1 : 0)>(a, o, Pin, Pout, dt, alpha, smem, m, out_slot != nullptr);
    else if (DIM >= 3)
      sweep_tile<T, DIM, RS, (DIM >= 3 ? 2 : 0)>(a, o, Pin, Pout, dt, alpha, smem, m, out_slot != nullptr);
  }
  if (out_slot) fold_maxima<DIM>(m, out_slot, red);
}

// ------------------------------------------------------------ magnetic sub-step

template <typename T>
__device__ __forceinline__ void cross3(const T* a, const T* b, T* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

// Loads the 3-vectors B and v at a (boundary-mapped) cell.  `Bs`/`vs` are
// either the iterate buffer (6 rows) or, for the first evaluation, the
// state's B rows and gas velocity rows (vz = 0 in 2D, _magnetic_field_update.py:60-70).
template <typename T, int DIM>
struct MagSrc {
  const T* B;   // 3 rows
  const T* v;   // DIM rows when `from_gas`, else 3 rows
  bool from_gas;
};

template <typename T, int DIM>
__device__ __forceinline__ void load_Bv(const MagSrc<T, DIM>& s, long long c, long long nc, T* B, T* v) {
  B[0] = s.B[c];
  B[1] = s.B[nc + c];
  B[2] = s.B[2 * nc + c];
  v[0] = s.v[c];
  v[1] = s.v[nc + c];
  v[2] = (DIM == 2 && s.from_gas) ? T(0) : s.v[2 * nc + c];
}

// The fields of FVArgs the point-wise magnetic work reads, copied into
// registers once per range of cells (read through the FVArgs reference, they
// would be reloaded after every global store, which may alias them).
template <typename T, int DIM>
struct MagCtx {
  T* state;
  long long nc;
  int n;
  T dx;
  bool midpoint;
  AxisMap<DIM> amap;
  __device__ __forceinline__ MagCtx(const FVArgs<T>& a, T* st)
      : state(st), nc(a.ncells), n(a.n), dx(T(a.dx)), midpoint(a.integrator == 0), amap(a) {}
  // the cell `off` cells away along axis k, boundary-mapped; *flip is set
  // when the cell is a reflective wall's mirror image
  __device__ __forceinline__ long long neighbor(const int* ic, int k, int off, bool* flip) const {
    int j[3] = {ic[0], ic[1], ic[2]};
    *flip = false;
    j[k] = amap(k, ic[k] + off, flip);
    return cell_index<DIM>(j[0], j[1], j[2], n);
  }
};

template <typename T, int DIM>
__device__ __forceinline__ void mag_direct_cell(const MagCtx<T, DIM>& x, const MagSrc<T, DIM>& src, T* dst, T dt,
                                                long long c, T& change) {
  const long long nc = x.nc;
  const int n = x.n;
  const T dx = x.dx;
  const MagSrc<T, DIM> s0{x.state + (DIM + 2) * nc, x.state + nc, true};  // B0, v0
  const T* rho = x.state;
  const bool midpoint = x.midpoint;
  int ic[3];
  if (DIM == 2) { ic[0] = (int)(c / n); ic[1] = (int)(c % n); ic[2] = 0; }
  else { ic[2] = (int)(c % n); ic[1] = (int)((c / n) % n); ic[0] = (int)(c / ((long long)n * n)); }
  // averaged fields at the cell and its 2*DIM neighbours
  T Bc[3], vc[3], B0c[3], v0c[3];
  // flip_c: the component of B and v that a reflective wall's ghost cell
  // negates -- the reference fills the 3-vectors with
  // _reflective_*_boundary(.., axis), which negates component `axis` (1
  // for x, 2 for y) rather than the wall-normal one (boundaries.py:324-355,
  // applied in _magnetic_field_update.py at every evaluation)
  auto avg_at = [&](long long cc, T* Ba, T* va, T* Bk_out, T* vk_out, T* B0_out, T* v0_out, int flip_c = -1) {
    T Bk[3], vk[3], B0[3], v0[3];
    load_Bv<T, DIM>(src, cc, nc, Bk, vk);
    load_Bv<T, DIM>(s0, cc, nc, B0, v0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const T sg = (i == flip_c) ? T(-1) : T(1);  // exact
      Bk[i] *= sg;
      vk[i] *= sg;
      B0[i] *= sg;
      v0[i] *= sg;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (midpoint) { Ba[i] = (Bk[i] + B0[i]) / T(2); va[i] = (vk[i] + v0[i]) / T(2); }
      else { Ba[i] = Bk[i]; va[i] = vk[i]; }
      if (Bk_out) { Bk_out[i] = Bk[i]; vk_out[i] = vk[i]; B0_out[i] = B0[i]; v0_out[i] = v0[i]; }
    }
  };
  T Ba_c[3], va_c[3];
  avg_at(c, Ba_c, va_c, Bc, vc, B0c, v0c);
  // E = cross(B, v) and B at neighbours; curls by central differences
  T Ep[3][3], Em[3][3], Bp[3][3], Bm[3][3];
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    T Ba[3], va[3];
    bool fl;
    const long long cp = x.neighbor(ic, k, +1, &fl);
    avg_at(cp, Ba, va, nullptr, nullptr, nullptr, nullptr, (fl && k + 1 < 3) ? k + 1 : -1);
    cross3(Ba, va, Ep[k]);
#pragma unroll
    for (int i = 0; i < 3; ++i) Bp[k][i] = Ba[i];
    const long long cm = x.neighbor(ic, k, -1, &fl);
    avg_at(cm, Ba, va, nullptr, nullptr, nullptr, nullptr, (fl && k + 1 < 3) ? k + 1 : -1);
    cross3(Ba, va, Em[k]);
#pragma unroll
    for (int i = 0; i < 3; ++i) Bm[k][i] = Ba[i];
  }
  // d(F_i)/d(x_k) = 0.5 (F_i[+] - F_i[-]) / dx
  auto dF = [&](T (*Fp)[3], T (*Fm)[3], int i, int k) { return T(0.5) * (Fp[k][i] - Fm[k][i]) / dx; };
  T curlE[3], curlB[3];
  if (DIM == 2) {
    curlE[0] = dF(Ep, Em, 2, 1);
    curlE[1] = -dF(Ep, Em, 2, 0);
    curlE[2] = dF(Ep, Em, 1, 0) - dF(Ep, Em, 0, 1);
    curlB[0] = dF(Bp, Bm, 2, 1);
    curlB[1] = -dF(Bp, Bm, 2, 0);
    curlB[2] = dF(Bp, Bm, 1, 0) - dF(Bp, Bm, 0, 1);
  } else {
    curlE[0] = dF(Ep, Em, 2, 1) - dF(Ep, Em, 1, 2);
    curlE[1] = dF(Ep, Em, 0, 2) - dF(Ep, Em, 2, 0);
    curlE[2] = dF(Ep, Em, 1, 0) - dF(Ep, Em, 0, 1);
    curlB[0] = dF(Bp, Bm, 2, 1) - dF(Bp, Bm, 1, 2);
    curlB[1] = dF(Bp, Bm, 0, 2) - dF(Bp, Bm, 2, 0);
    curlB[2] = dF(Bp, Bm, 1, 0) - dF(Bp, Bm, 0, 1);
  }
  T phi2[3];
  cross3(Ba_c, curlB, phi2);
  const T r = rho[c];
  T Bn[3], vn[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Bn[i] = B0c[i] - dt * curlE[i];
    vn[i] = v0c[i] - dt * (phi2[i] / r);
  }
  const T dB = Num<T>::sqrt_(sq(Bc[0] - Bn[0]) + sq(Bc[1] - Bn[1]) + sq(Bc[2] - Bn[2]));
  const T dv = Num<T>::sqrt_(sq(vc[0] - vn[0]) + sq(vc[1] - vn[1]) + sq(vc[2] - vn[2]));
  change = nanmax(change, nanmax(dB, dv));
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    dst[i * nc + c] = Bn[i];
    dst[(3 + i) * nc + c] = vn[i];
  }
}

// One evaluation of the fixed-point map without shared memory: every cell
// gathers the averaged fields of its 2*DIM neighbours itself (L1 serves the
// reuse).  Used when the state is L2-resident (2D), where the tiled variant
// below loses more to tile imbalance and barriers than it saves in loads.
template <typename T, int DIM>
__device__ __noinline__ void phase_mag_iterate_direct(const FVArgs<T>& a, T* state, MagSrc<T, DIM> src, T* dst,
                                                      T dt, unsigned long long* slot, double* red) {
  const long long nc = a.ncells;
  T change = T(0);
  MagItems<T, DIM>::direct(a, state, src, dst, dt, (long long)blockIdx.x * blockDim.x + threadIdx.x, nc,
                           (long long)gridDim.x * blockDim.x, &change);
  const double r = block_max<double>((double)change, red);
  if (threadIdx.x == 0) atomic_max_nonneg(slot, r);
}

// B and v iterates: `Bk`/`vk` are the iterate buffer rows, or null for the
// first evaluation, which starts from B0 and v0 (the state's B rows and gas
// velocity, vz = 0 in 2D as in _magnetic_field_update.py:60-70).
template <typename T, int DIM>
__device__ __forceinline__ void load_iter(const T* st, const T* src, long long c, long long nc, T* Bk,
                                          T* vk, T* B0, T* v0) {
  B0[0] = st[(DIM + 2) * nc + c];
  B0[1] = st[(DIM + 3) * nc + c];
  B0[2] = st[(DIM + 4) * nc + c];
  v0[0] = st[nc + c];
  v0[1] = st[2 * nc + c];
  v0[2] = (DIM == 3) ? st[3 * nc + c] : T(0);
  if (src) {
#pragma unroll
    for (int i = 0; i < 3; ++i) { Bk[i] = src[i * nc + c]; vk[i] = src[(3 + i) * nc + c]; }
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) { Bk[i] = B0[i]; vk[i] = v0[i]; }
  }
}

// One evaluation of the fixed-point map (_magnetic_field_update.py:82-105,
// :143-165): B_{k+1} = B0 - dt curl(B x v), v_{k+1} = v0 - dt (B x curl B)/rho
// with B, v the averages (midpoint) or the iterate (Euler).  A halo-1 tile of
// the averaged B and of E = B x v is staged in shared memory, so every cell
// computes its cross product once.  Folds max |B_k - B_{k+1}| and
// max |v_k - v_{k+1}| into `slot`.
template <typename T, int DIM, int V = 0>
__device__ __forceinline__ void mag_tile(const FVArgs<T>& a, const T* state, const int* o, const T* src, T* dst,
                                         T dt, T* smem, T* change_io) {
  using G = TileGeom<T, DIM, V>;
  const long long nc = a.ncells;
  const int n = a.n;
  const T dx = T(a.dx);
  const T hdx = T(0.5 * a.inv_dx);
  const bool midpoint = (a.integrator == 0);
  const AxisMap<DIM> amap(a);
  T* sB = smem;                 // [3][MHALO] averaged B
  T* sE = smem + 3 * G::MHALO;  // [3][MHALO] E = B x v
  T change = *change_io;
  for (int e = threadIdx.x; e < G::MHALO; e += blockDim.x) {
    const int h2 = e % G::M2, h1 = (e / G::M2) % G::M1, h0 = e / (G::M2 * G::M1);
    bool fl = false;
    const int i0 = amap(0, o[0] + h0 - 1, &fl);
    const int i1 = amap(1, o[1] + h1 - 1, &fl);
    const int i2 = (DIM >= 3) ? amap(2, o[2] + h2 - 1, &fl) : 0;
    const long long c = cell_index<DIM>(i0, i1, i2, n);
    T Bk[3], vk[3], B0[3], v0[3], Ba[3], va[3], E[3];
    load_iter<T, DIM>(state, src, c, nc, Bk, vk, B0, v0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      Ba[i] = midpoint ? (Bk[i] + B0[i]) / T(2) : Bk[i];
      va[i] = midpoint ? (vk[i] + v0[i]) / T(2) : vk[i];
    }
    cross3(Ba, va, E);
#pragma unroll
    for (int i = 0; i < 3; ++i) { sB[i * G::MHALO + e] = Ba[i]; sE[i * G::MHALO + e] = E[i]; }
  }
  __syncthreads();
  for (int cl = threadIdx.x; cl < G::CELLS; cl += blockDim.x) {
    const int c2 = cl % G::T2, c1 = (cl / G::T2) % G::T1, c0 = cl / (G::T2 * G::T1);
    const int g0 = o[0] + c0, g1 = o[1] + c1, g2 = o[2] + c2;
    if (g0 >= n || g1 >= n || (DIM >= 3 && g2 >= n)) continue;
    const long long c = cell_index<DIM>(g0, g1, g2, n);
    const int h = ((c0 + 1) * G::M1 + (c1 + 1)) * G::M2 + (DIM >= 3 ? c2 + 1 : 0);
    const int st[3] = {G::M1 * G::M2, G::M2, 1};
    // d(F_i)/d(x_k) = 0.5 (F_i[+] - F_i[-]) / dx  (_vector_maths.py:55-100);
    // FP32 multiplies by 0.5 / dx instead of dividing
    auto dF = [&](const T* F, int i, int k) {
      const T d = F[i * G::MHALO + h + st[k]] - F[i * G::MHALO + h - st[k]];
      if constexpr (sizeof(T) == 4) return d * hdx;
      else return T(0.5) * d / dx;
    };
    T curlE[3], curlB[3];
    if (DIM == 2) {
      curlE[0] = dF(sE, 2, 1);
      curlE[1] = -dF(sE, 2, 0);
      curlE[2] = dF(sE, 1, 0) - dF(sE, 0, 1);
      curlB[0] = dF(sB, 2, 1);
      curlB[1] = -dF(sB, 2, 0);
      curlB[2] = dF(sB, 1, 0) - dF(sB, 0, 1);
    } else {
      curlE[0] = dF(sE, 2, 1) - dF(sE, 1, 2);
      curlE[1] = dF(sE, 0, 2) - dF(sE, 2, 0);
      curlE[2] = dF(sE, 1, 0) - dF(sE, 0, 1);
      curlB[0] = dF(sB, 2, 1) - dF(sB, 1, 2);
      curlB[1] = dF(sB, 0, 2) - dF(sB, 2, 0);
      curlB[2] = dF(sB, 1, 0) - dF(sB, 0, 1);
    }
    T Bk[3], vk[3], B0[3], v0[3], Ba[3];
    load_iter<T, DIM>(state, src, c, nc, Bk, vk, B0, v0);
#pragma unroll
    for (int i = 0; i < 3; ++i) Ba[i] = sB[i * G::MHALO + h];
    T phi2[3];
    cross3(Ba, curlB, phi2);
    const T r = state[c];
    T Bn[3], vn[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      Bn[i] = B0[i] - dt * curlE[i];
      vn[i] = v0[i] - dt * (phi2[i] / r);
    }
    const T dB = Num<T>::sqrt_(sq(Bk[0] - Bn[0]) + sq(Bk[1] - Bn[1]) + sq(Bk[2] - Bn[2]));
    const T dv = Num<T>::sqrt_(sq(vk[0] - vn[0]) + sq(vk[1] - vn[1]) + sq(vk[2] - vn[2]));
    change = nanmax(change, nanmax(dB, dv));
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dst[i * nc + c] = Bn[i];
      dst[(3 + i) * nc + c] = vn[i];
    }
  }
  __syncthreads();
  *change_io = change;
}

// A cell's inputs to one evaluation of the fixed-point map.
template <typename T>
struct MagRaw {
  T Bk[3], vk[3], B0[3], v0[3];
};

// Planes per work item of mag_stream: the run length that minimises (rounds of
// work items over the grid) x (planes staged per item, the run plus two).
__device__ __forceinline__ int mag_stream_run(int n, int grid) {
  const long long cols = (long long)((n + kMS1 - 1) / kMS1) * ((n + kMS2 - 1) / kMS2);
  int best = n;
  long long best_cost = -1;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int c = (i == 7) ? n : (8 << (i / 2)) + ((i & 1) ? (4 << (i / 2)) : 0);  // 8 12 16 24 32 48 64, n
    const int L = c < n ? c : n;
    const long long items = cols * ((n + L - 1) / L);
    const long long cost = ((items + grid - 1) / grid) * (L + 2);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = L;
    }
  }
  return best;
}

// One 3D evaluation of the fixed-point map with the arithmetic of mag_tile,
// streamed along axis 0 (FP32).  A work item is a column of kMS1 x kMS2 cells
// (axes 1, 2) over a run of planes; the averaged B and E = B x v of four
// consecutive planes, each with its axis-1/2 halo (no corners: the curls read
// no diagonal neighbour), sit in a shared-memory ring.  Each thread loads its
// own cell's inputs once, two planes before the plane is updated, and parks
// them in shared memory for the update: a cell's fields are read once per
// evaluation (plus the halo of the column and two planes per run) instead of
// once per halo-1 tile that covers it (2.4 times with 4 x 4 x 32 tiles).  The
// rows of the plane AMX_MAG_PF planes ahead are prefetched into L2.
template <typename T>
__device__ __forceinline__ void mag_stream(const FVArgs<T>& a, const T* state, const T* src, T* dst, T dt,
                                           T* ring, T* change_io) {
  T* raw = ring + 4 * 6 * kMSP;  // [2][kMSRaw][kFVThreads]
  const long long nc = a.ncells;
  const int n = a.n;
  const T dx = T(a.dx);
  const T hdx = T(0.5 * a.inv_dx);
  const bool midpoint = (a.integrator == 0);
  const AxisMap<3> amap(a);
  const int L = mag_stream_run(n, gridDim.x);
  const int C1 = (n + kMS1 - 1) / kMS1, C2 = (n + kMS2 - 1) / kMS2;
  const long long items = (long long)C1 * C2 * ((n + L - 1) / L);
  const int t = threadIdx.x;
  const int c1 = t / kMS2, c2 = t % kMS2;
  const int hOwn = (c1 + 1) * kMSW2 + (c2 + 1);
  // this thread's halo entry (threads below kMSRing): the rows beside the
  // tile along axis 1, then the columns beside it along axis 2
  const bool has_ring = t < kMSRing;
  int r1, r2;
  if (t < kMS2) { r1 = -1; r2 = t; }
  else if (t < 2 * kMS2) { r1 = kMS1; r2 = t - kMS2; }
  else if (t < 2 * kMS2 + kMS1) { r1 = t - 2 * kMS2; r2 = -1; }
  else { r1 = t - 2 * kMS2 - kMS1; r2 = kMS2; }
  const int hRing = (r1 + 1) * kMSW2 + (r2 + 1);
  // the row this thread prefetches into L2 for a plane: threads below 13 x
  // kMS1 take the tile's rows of the 13 input arrays (B0, v0, iterate B and
  // v, density), the next 24 the two halo rows of the 12 vector arrays
  int pa = -1, pr = 0;
  if (t < kMSRaw * kMS1) { pa = t / kMS1; pr = t % kMS1; }
  else if (t < kMSRaw * kMS1 + 24) { const int u = t - kMSRaw * kMS1; pa = u >> 1; pr = (u & 1) ? kMS1 : -1; }
  const T* parr = nullptr;
  if (pa >= 0 && pa < 3) parr = state + (5 + pa) * nc;
  else if (pa >= 3 && pa < 6) parr = state + (1 + pa - 3) * nc;
  else if (pa >= 6 && pa < 12) parr = src ? src + (pa - 6) * nc : nullptr;
  else if (pa == 12) parr = state;
  T change = *change_io;

  auto load = [&](long long c, MagRaw<T>& r) { load_iter<T, 3>(state, src, c, nc, r.Bk, r.vk, r.B0, r.v0); };
  // the own cell's inputs of plane q into raw slot q & 1
  auto park = [&](int sl, const MagRaw<T>& r, T rho) {
    T* d = raw + sl * (kMSRaw * kFVThreads) + t;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      d[(0 + i) * kFVThreads] = r.Bk[i];
      d[(3 + i) * kFVThreads] = r.vk[i];
      d[(6 + i) * kFVThreads] = r.B0[i];
      d[(9 + i) * kFVThreads] = r.v0[i];
    }
    d[12 * kFVThreads] = rho;
  };
  auto put = [&](T* sl, int h, const MagRaw<T>& r) {
    T Ba[3], va[3], E[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      Ba[i] = midpoint ? (r.Bk[i] + r.B0[i]) / T(2) : r.Bk[i];
      va[i] = midpoint ? (r.vk[i] + r.v0[i]) / T(2) : r.vk[i];
    }
    cross3(Ba, va, E);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      sl[i * kMSP + h] = Ba[i];
      sl[(3 + i) * kMSP + h] = E[i];
    }
  };

  for (long long item = blockIdx.x; item < items; item += gridDim.x) {
    const int t2 = (int)(item % C2);
    const int t1 = (int)((item / C2) % C1);
    const int lo = (int)(item / ((long long)C2 * C1)) * L;
    const int hi = lo + L < n ? lo + L : n;
    const int g1 = t1 * kMS1 + c1, g2 = t2 * kMS2 + c2;
    const bool valid = g1 < n && g2 < n;
    bool fl;
    const int j1 = amap(1, g1, &fl), j2 = amap(2, g2, &fl);
    const int k1 = amap(1, t1 * kMS1 + r1, &fl), k2 = amap(2, t2 * kMS2 + r2, &fl);
    auto own_cell = [&](int q) { return cell_index<3>(amap(0, q, &fl), j1, j2, n); };
    auto ring_cell = [&](int q) { return cell_index<3>(amap(0, q, &fl), k1, k2, n); };
    auto slot = [&](int q) { return ring + ((q - lo + 1) & 3) * (6 * kMSP); };
    const int pj1 = amap(1, t1 * kMS1 + pr, &fl);
    auto prefetch = [&](int q) {
      if (AMX_MAG_PF > 0 && parr && q <= hi)
        asm volatile("prefetch.L2 [%0];" ::"l"(parr + cell_index<3>(amap(0, q, &fl), pj1, t2 * kMS2, n)));
    };
#pragma unroll 1
    for (int q = lo + 2; q < lo + AMX_MAG_PF; ++q) prefetch(q);

    MagRaw<T> R, Q;
    T rho = T(0);
    // planes lo - 1, lo, lo + 1 (hi >= lo + 1: every run has a plane)
#pragma unroll 1
    for (int q = lo - 1; q <= lo + 1; ++q) {
      const long long c = own_cell(q);
      load(c, R);
      if (q >= lo) rho = state[c];
      if (has_ring) load(ring_cell(q), Q);
      put(slot(q), hOwn, R);
      if (has_ring) put(slot(q), hRing, Q);
      if (q >= lo) park((q - lo) & 1, R, rho);
    }
    __syncthreads();

#pragma unroll 1
    for (int p = lo; p < hi; ++p) {
      prefetch(p + AMX_MAG_PF);
      const bool more = p + 2 <= hi;
      if (valid) {
        const T* r0 = raw + ((p - lo) & 1) * (kMSRaw * kFVThreads) + t;
        const T* Sm = slot(p - 1);
        const T* S0 = slot(p);
        const T* Sp = slot(p + 1);
        // d(F_i)/d(x_k) = 0.5 (F_i[+] - F_i[-]) / dx  (_vector_maths.py:55-100);
        // FP32 multiplies by 0.5 / dx instead of dividing
        auto dF = [&](int f, int i, int k) {
          const int o = (f + i) * kMSP + hOwn;
          const T d = (k == 0) ? Sp[o] - Sm[o] : (k == 1) ? S0[o + kMSW2] - S0[o - kMSW2] : S0[o + 1] - S0[o - 1];
          if constexpr (sizeof(T) == 4) return d * hdx;
          else return T(0.5) * d / dx;
        };
        T curlE[3], curlB[3];
        curlE[0] = dF(3, 2, 1) - dF(3, 1, 2);
        curlE[1] = dF(3, 0, 2) - dF(3, 2, 0);
        curlE[2] = dF(3, 1, 0) - dF(3, 0, 1);
        curlB[0] = dF(0, 2, 1) - dF(0, 1, 2);
        curlB[1] = dF(0, 0, 2) - dF(0, 2, 0);
        curlB[2] = dF(0, 1, 0) - dF(0, 0, 1);
        T Ba[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) Ba[i] = S0[i * kMSP + hOwn];
        T phi2[3];
        cross3(Ba, curlB, phi2);
        const T rho0 = r0[12 * kFVThreads];
        T Bn[3], vn[3], dBs[3], dvs[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          Bn[i] = r0[(6 + i) * kFVThreads] - dt * curlE[i];
          vn[i] = r0[(9 + i) * kFVThreads] - dt * (phi2[i] / rho0);
          dBs[i] = r0[(0 + i) * kFVThreads] - Bn[i];
          dvs[i] = r0[(3 + i) * kFVThreads] - vn[i];
        }
        const T dB = Num<T>::sqrt_(sq(dBs[0]) + sq(dBs[1]) + sq(dBs[2]));
        const T dv = Num<T>::sqrt_(sq(dvs[0]) + sq(dvs[1]) + sq(dvs[2]));
        change = nanmax(change, nanmax(dB, dv));
        const long long c = cell_index<3>(p, g1, g2, n);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          dst[i * nc + c] = Bn[i];
          dst[(3 + i) * nc + c] = vn[i];
        }
      }
      // the inputs of plane p + 2, after the update of plane p (loading them
      // before it, to overlap, spills at this kernel's 80 registers and
      // measured slower); the L2 prefetch above hides their memory latency
      if (more) {
        const long long c = own_cell(p + 2);
        load(c, R);
        rho = state[c];
        if (has_ring) load(ring_cell(p + 2), Q);
        put(slot(p + 2), hOwn, R);
        if (has_ring) put(slot(p + 2), hRing, Q);
        park((p + 2 - lo) & 1, R, rho);  // the slot plane p's inputs leave
      }
      __syncthreads();
    }
  }
  *change_io = change;
}

template <typename T, int DIM>
__device__ __noinline__ void phase_mag_iterate(const FVArgs<T>& a, const T* state, const T* src, T* dst, T dt,
                                               unsigned long long* slot, double* red, T* smem) {
  T change = T(0);
  if constexpr (DIM == 3 && sizeof(T) == 4) {
    mag_stream<T>(a, state, src, dst, dt, smem, &change);
  } else {
    using G = TileGeom<T, DIM>;
    const long long ntiles = fv_num_tiles<DIM>(a.n, G::T0, G::T1, G::T2);
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
      int o[3];
      tile_origin<DIM>(tile, a.n, G::T0, G::T1, G::T2, o);
      mag_tile<T, DIM>(a, state, o, src, dst, dt, smem, &change);
    }
  }
  const double r = block_max<double>((double)change, red);
  if (threadIdx.x == 0) atomic_max_nonneg(slot, r);
}

// Pressure refresh with gamma = 5/3 and write-back of one cell
// (_magnetic_field_update.py:208-242) from `state` into `out` (the same
// array, or a copy that also receives the density); tracks |u_a| + c of the
// updated gas.
template <typename T, int DIM>
__device__ __forceinline__ void mag_finalize_cell(const T* state, T* out, long long nc, T gamma, const T* Bv,
                                                  long long c, bool track, T* m) {
  const T g53 = T(5.0 / 3.0);
  const T rho = state[c];
  const T p = state[(DIM + 1) * nc + c];
  T v0[3];
  v0[0] = state[nc + c];
  v0[1] = state[2 * nc + c];
  v0[2] = (DIM == 3) ? state[3 * nc + c] : T(0);
  T vn[3], Bn[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) { Bn[i] = Bv[i * nc + c]; vn[i] = Bv[(3 + i) * nc + c]; }
  const T v0abs = Num<T>::sqrt_(v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
  const T vnabs = Num<T>::sqrt_(vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2]);
  T E = total_energy(rho, v0abs, p, g53);
  E = E - T(0.5) * rho * (v0abs * v0abs) + T(0.5) * rho * (vnabs * vnabs);
  const T pn = pressure_from_energy(E, rho, vnabs, g53);
  T q[DIM + 2];
  q[0] = rho;
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    out[(1 + i) * nc + c] = vn[i];
    q[1 + i] = vn[i];
  }
  out[(DIM + 1) * nc + c] = pn;
  q[DIM + 1] = pn;
#pragma unroll
  for (int i = 0; i < 3; ++i) out[(DIM + 2 + i) * nc + c] = Bn[i];
  if (out != state) out[c] = rho;
  if (track) track_maxima<T, DIM>(q, gamma, m);
}

// ------------------------------------------------------------ per-item entry points

// The work items of the FV step as the single-run and the batched kernels
// call them: one hydro tile, and a strided range of cells of the fixed-point
// map or of the write-back.  Where they are separate (not inlined)
// functions, every kernel executes the same compiled arithmetic: branches
// (IEEE division, data-dependent selects) let the compiler fuse
// multiply-adds differently in different callers.  The FP32 hydro tile
// (approximate division, straight-line code) is inlined and gives identical
// results all the same.
template <typename T, int DIM, int RS, int V>
struct FVItems {
  template <bool PP = false>
  static __device__ __forceinline__ void hydro(const FVArgs<T>& a, const int* o, const T* Pin, T* Pout,
                                               const T* P0, T dt, const T* alpha, T* smem, T* m, bool track,
                                               const T* ppC = nullptr) {
    hydro_tile<T, DIM, RS, V, PP>(a, o, Pin, Pout, P0, dt, alpha, smem, m, track, ppC);
  }
};
template <int DIM, int RS, int V>
struct FVItems<double, DIM, RS, V> {
  template <bool PP = false>
  static __device__ __noinline__ void hydro(const FVArgs<double>& a, const int* o, const double* Pin, double* Pout,
                                            const double* P0, double dt, const double* alpha, double* smem,
                                            double* m, bool track, const double* ppC = nullptr) {
    hydro_tile<double, DIM, RS, V, PP>(a, o, Pin, Pout, P0, dt, alpha, smem, m, track, ppC);
  }
};

// The magnetic items are separate functions in both precisions: the
// reflective walls' sign flips put data-dependent selects into the map.
template <typename T, int DIM>
struct MagItems {
  static __device__ __noinline__ void direct(const FVArgs<T>& a, T* state, const MagSrc<T, DIM>& src, T* dst, T dt,
                                             long long c, long long end, long long step, T* change) {
    const MagCtx<T, DIM> x(a, state);
    T ch = *change;
    for (; c < end; c += step) mag_direct_cell<T, DIM>(x, src, dst, dt, c, ch);
    *change = ch;
  }
  static __device__ __noinline__ void finalize(const FVArgs<T>& a, const T* state, const T* Bv, T* out, long long c,
                                               long long end, long long step, bool track, T* m) {
    const long long nc = a.ncells;
    const T gamma = T(a.gamma);
    for (; c < end; c += step) mag_finalize_cell<T, DIM>(state, out, nc, gamma, Bv, c, track, m);
  }
};

// The write-back phase over all cells; folds the maxima of |u_a| + c of the
// updated gas into `out_slot` when given.
template <typename T, int DIM>
__device__ __noinline__ void phase_mag_finalize(const FVArgs<T>& a, const T* state, const T* Bv, T* out,
                                                unsigned long long* out_slot, double* red) {
  const long long nc = a.ncells;
  T m[3] = {T(0), T(0), T(0)};
  MagItems<T, DIM>::finalize(a, state, Bv, out, (long long)blockIdx.x * blockDim.x + threadIdx.x, nc,
                             (long long)gridDim.x * blockDim.x, out_slot != nullptr, m);
  if (out_slot) fold_maxima<DIM>(m, out_slot, red);
}

// ------------------------------------------------------------ the kernel

// 3D is bound by HBM latency: its FP32 instantiations are held to three resident
// blocks per SM (85 registers), 1D and 2D to two (128 registers).
// SCHEME: FV_UNSPLIT, FV_SPLIT (MUSCL-Hancock sweeps) or FV_UNSPLIT_PP
// (VAN_ALBADA_PP reconstruction); a compile-time choice, so that the
// ordinary scheme's kernel carries none of the others' code.
template <typename T, int DIM, int RS, bool MHD, int SCHEME = FV_UNSPLIT>
__global__ void __launch_bounds__(kFVThreads, (DIM == 3 && sizeof(T) == 4) ? 3 : 2)
fv_run_kernel(FVArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  __shared__ double red[32];
  FVControl* ctl = a.ctl;
  int* status = &ctl->status;
  const GridBarrier bar{&ctl->bar_count, &ctl->abort_flag, a.spin_limit};
  const long long nc = a.ncells;
  T* gas = a.state;
  constexpr int NVG_ = DIM + 2;
  __shared__ T s_alpha[3];
  __shared__ T s_ppC[3];
  // VAN_ALBADA_PP (unsplit): every stage needs C_k from the maxima of its input
  constexpr bool pp = (SCHEME == FV_UNSPLIT_PP) && DIM >= 2;
  constexpr bool split = (SCHEME == FV_SPLIT);

  // Producer ring of maxima: the phase with pass number rp writes slot rp % 3
  // after block 0 cleared slot (rp + 1) % 3; the slot a phase reads is the
  // one written by the previous producer, (rp - 1) % 3.
  int rp = 0, mag_pass = 0;

  auto produce_slot = [&]() -> unsigned long long* {
    if (blockIdx.x == 0 && threadIdx.x < 4) ctl->red[(rp + 1) % 3][threadIdx.x] = 0ull;
    return ctl->red[rp % 3];
  };
  auto last_maxima = [&](double* m) {
    volatile unsigned long long* s = ctl->red[(rp + 2) % 3];
#pragma unroll
    for (int k = 0; k < 3; ++k) m[k] = (k < DIM) ? bits_to_double(s[k]) : 0.0;
  };
  auto set_alpha = [&]() {
    if (RS != RS_LF && !pp) return;
    double m[3];
    last_maxima(m);
    if (RS == RS_LF && threadIdx.x < DIM) s_alpha[threadIdx.x] = T(m[threadIdx.x]);
    if (pp && threadIdx.x == 0) {  // (pp is a compile-time constant)
      // C = alpha_lax / sum(alpha_lax) (reconstruction.py:172-182)
      T tot = T(m[0]);
#pragma unroll
      for (int k = 1; k < DIM; ++k) tot = tot + T(m[k]);
#pragma unroll
      for (int k = 0; k < DIM; ++k) s_ppC[k] = T(m[k]) / tot;
    }
    __syncthreads();
  };
  // `need`: whether anything reads the maxima of this stage's output (the
  // next stage's Lax-Friedrichs alpha, or the next step's dt)
  auto stage = [&](const T* in, T* out, const T* p0, T h, bool need) -> bool {
    set_alpha();
    unsigned long long* slot = produce_slot();
    if constexpr (pp) {
      phase_hydro_stage<T, DIM, RS, true>(a, in, out, p0, h, RS == RS_LF ? s_alpha : nullptr, smem, slot, red,
                                          s_ppC);
    } else {
      phase_hydro_stage<T, DIM, RS>(a, in, out, p0, h, RS == RS_LF ? s_alpha : nullptr, smem,
                                    (need || RS == RS_LF) ? slot : nullptr, red);
    }
    ++rp;
    return grid_sync(bar, status);
  };
  // one RK2 update of the gas rows with stage dt `h` (evolve_state.py:419-488);
  // `last`: the update ends the time step
  auto rk2_unsplit = [&](T h, bool last) -> bool {
    if (!stage(gas, a.p1, nullptr, h, false)) return false;
    return stage(a.p1, gas, gas, h, last);
  };
  // one split sweep along axis k (evolve_state.py:52-160)
  auto sweep = [&](const T* in, T* out, int k, T h, bool need) -> bool {
    set_alpha();
    unsigned long long* slot = produce_slot();
    if constexpr (split)
      phase_sweep<T, DIM, RS>(a, k, in, out, h, RS == RS_LF ? s_alpha : nullptr, smem,
                              (need || RS == RS_LF) ? slot : nullptr, red);
    ++rp;
    return grid_sync(bar, status);
  };
  // _evolve_gas_state_split (evolve_state.py:168-325): Strang sequence of
  // sweeps x(h/2) y(h) x(h/2) in 2D, x(h/2) y(h/2) z(h) y(h/2) x(h/2) in 3D,
  // rotating through the state, p1 and p2 so that the last one lands in the
  // state; in 1D the single sweep's result is copied back
  auto split_update = [&](T h, bool last) -> bool {
    if constexpr (!split) {
      return false;
    } else {
    if (DIM == 1) {
      if (!sweep(gas, a.p1, 0, h, last)) return false;
      const long long total = (long long)NVG_ * nc;
      for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
           e += (long long)gridDim.x * blockDim.x)
        gas[e] = a.p1[e];
      return grid_sync(bar, status);
    }
    const T h2 = h / T(2);
    if (DIM == 2) {
      if (!sweep(gas, a.p1, 0, h2, false)) return false;
      if (!sweep(a.p1, a.p2, 1, h, false)) return false;
      return sweep(a.p2, gas, 0, h2, last);
    }
    if (!sweep(gas, a.p1, 0, h2, false)) return false;
    if (!sweep(a.p1, a.p2, 1, h2, false)) return false;
    if (!sweep(a.p2, a.p1, 2, h, false)) return false;
    if (!sweep(a.p1, a.p2, 1, h2, false)) return false;
    return sweep(a.p2, gas, 0, h2, last);
    }
  };
  // the gas update of the configured scheme
  auto rk2 = [&](T h, bool last) -> bool {
    if constexpr (split) return split_update(h, last);
    else return rk2_unsplit(h, last);
  };

  // magnetic_update (_magnetic_field_update.py:37-242); returns iterations or -1.
  // Per cell (mag_direct_cell) in 2D, and in 3D with a reflective wall, whose
  // ghost cells of the B and v 3-vectors negate component `axis` of the wall
  // (boundaries.py:324-355: y at x walls, z at y walls, and at z walls a
  // fourth component, an update JAX drops); tiled or streamed otherwise.
  const bool mag_direct = (DIM == 2) || (DIM == 3 && AxisMap<DIM>(a).reflective);
  auto magnetic = [&](T h) -> int {
    unsigned long long* slot = &ctl->mag[mag_pass % 3];
    if (mag_direct) {
      const MagSrc<T, DIM> first{gas + (DIM + 2) * nc, gas + nc, true};
      phase_mag_iterate_direct<T, DIM>(a, gas, first, a.mag0, h, slot, red);
    } else {
      phase_mag_iterate<T, DIM>(a, gas, nullptr, a.mag0, h, slot, red, smem);
    }
    if (!grid_sync(bar, status)) return -1;
    double change = bits_to_double(*(volatile unsigned long long*)slot);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag[(mag_pass + 2) % 3] = 0ull;
    ++mag_pass;
    int it = 0;
    T* cur = a.mag0;
    T* nxt = a.mag1;
    while (change > a.tol && it < a.max_iters) {
      slot = &ctl->mag[mag_pass % 3];
      if (mag_direct) {
        const MagSrc<T, DIM> src{cur, cur + 3 * nc, false};
        phase_mag_iterate_direct<T, DIM>(a, gas, src, nxt, h, slot, red);
      } else {
        phase_mag_iterate<T, DIM>(a, gas, cur, nxt, h, slot, red, smem);
      }
      if (!grid_sync(bar, status)) return -1;
      change = bits_to_double(*(volatile unsigned long long*)slot);
      if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag[(mag_pass + 2) % 3] = 0ull;
      ++mag_pass;
      ++it;
      T* tmp = cur; cur = nxt; nxt = tmp;
    }
    if (change > a.tol && blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, AMX_ERR_NOT_CONVERGED);
    if (change != change && blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, AMX_ERR_NAN);
    unsigned long long* out = produce_slot();
    phase_mag_finalize<T, DIM>(a, gas, cur, gas, (RS == RS_LF || pp) ? out : nullptr, red);
    ++rp;
    if (!grid_sync(bar, status)) return -1;
    return it;
  };

  // CFL dt from the maxima of the last producer (_timestep_estimator.py:118-128)
  // (split: _timestep_estimator.py:130-218, the largest |u_a| + c over all
  // axes, dt = C dx / w, clamped to dt_max when use_max_adaptive_timestep)
  auto dt_from_maxima = [&]() -> double {
    double m[3];
    last_maxima(m);
    if constexpr (split) {
      double w = m[0];
#pragma unroll
      for (int k = 1; k < DIM; ++k) w = nanmax(w, m[k]);
      double dt = a.C_cfl * a.dx / w;
      if (a.use_dt_max) dt = nanmin(dt, a.dt_max);
      return dt;
    }
    double sum = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) sum = (k == 0) ? m[k] / a.dx : sum + m[k] / a.dx;
    return a.C_cfl * 1.0 / sum;
  };
  auto cfl_phase = [&]() -> bool {
    unsigned long long* slot = produce_slot();
    phase_cfl<T, DIM>(a, gas, slot, red);
    ++rp;
    return grid_sync(bar, status);
  };

  if (a.mode == FV_MODE_CFL) {
    if (!cfl_phase()) return;
    const double dt = dt_from_maxima();
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->dt = dt;
    return;
  }
  // The dt of the next step of a device-driven step sequence (the step loop
  // of time_integration.py:626-677): no step once t reached t_end (adaptive
  // dt), t_pause or an error; otherwise the CFL dt (or the fixed one),
  // clipped to the end time.  Every block reads the same t and status.
  if (a.mode == FV_MODE_DT) {
    const double t = *(volatile double*)&ctl->t;
    const int st = *(volatile int*)status;
    bool go = !(t >= a.t_pause) && !(st & (AMX_ERR_TIMEOUT | AMX_ERR_NAN));
    if (!a.fixed_timestep && !(t < a.t_end)) go = false;
    if (!go) {
      if (blockIdx.x == 0 && threadIdx.x == 0) ctl->active = 0;
      return;
    }
    if (!cfl_phase()) return;
    double dt = a.fixed_timestep ? a.dt_fixed : dt_from_maxima();
    if (a.exact_end_time) dt = nanmin(dt, a.t_end - t);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (dt != dt) raise_status(status, AMX_ERR_NAN);
      ctl->dt = dt;
      ctl->active = 1;
    }
    return;
  }
  // the seams need the maxima of the state they start from only for the
  // Lax-Friedrichs alpha and the VAN_ALBADA_PP weights
  constexpr bool seam_maxima = (RS == RS_LF) || pp;
  if (a.mode == FV_MODE_HYDRO_RK2) {
    double dt_in = a.dt_in;
    if (a.dt_dev) {
      if (!*(volatile int*)&ctl->active) return;
      dt_in = *(volatile double*)&ctl->dt;
    }
    if (seam_maxima) {
      if (!cfl_phase()) return;
      // the gravity source term's Lax-Friedrichs alpha (the old state's maxima)
      if (a.dt_dev && blockIdx.x == 0 && threadIdx.x == 0) {
        double m[3];
        last_maxima(m);
        for (int k = 0; k < 3; ++k) ctl->seam_maxima[k] = m[k];
      }
    }
    rk2(T(dt_in * a.dt_scale), false);
    return;
  }
  if (a.mode == FV_MODE_MAGNETIC) {
    if (!MHD) return;
    double dt_in = a.dt_in;
    if (a.dt_dev) {
      if (!*(volatile int*)&ctl->active) return;
      dt_in = *(volatile double*)&ctl->dt;
    }
    const int it = magnetic(T(dt_in));
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag_iters = it;
    return;
  }
  if (a.mode == FV_MODE_EVOLVE) {
    double dt_in = a.dt_in;
    if (a.dt_dev) {
      if (!*(volatile int*)&ctl->active) return;
      dt_in = *(volatile double*)&ctl->dt;
    }
    if (seam_maxima && !cfl_phase()) return;
    const T dtT = T(dt_in);
    if (MHD) {
      if (!rk2(dtT / T(2), false)) return;
      const int it = magnetic(dtT);
      if (it < 0) return;
      if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag_iters = it;
      rk2(dtT / T(2), false);
    } else {
      rk2(dtT, false);
    }
    return;
  }

  // ---- full time steps (time_integration.py:386-762)
  //
  // Tape mode keeps every intermediate state: the step starting at element
  // offset `toff` of the tape lays out, in rows of ncells values,
  //   S0 (NVT rows: the step's start state), S1 (NVG: stage 1),
  //   MHD: S2 (NVT: stage 2 gas rows, B rows of S0), Z0..Zk (6 rows each:
  //        the fixed-point iterates), S3 (NVT: after the write-back),
  //        S4 (NVG: stage 3),
  //   S5 (NVT: the end state) = the next step's S0,
  // and tape_off[step + 1] records where S5 starts.  A step that would not
  // fit stops the run with AMX_ERR_TOO_LARGE.
  constexpr int NVG = DIM + 2, NVT = DIM + 2 + (MHD ? 3 : 0);
  const bool taping = a.tape != nullptr;
  const long long step0 = *(volatile long long*)&ctl->steps;
  long long toff = 0;
  if (taping) {
    if (step0 > a.max_hist) {
      if (blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, AMX_ERR_TOO_LARGE);
      return;
    }
    toff = *(volatile long long*)&a.tape_off[step0];
  }
  // copies `rows` rows (all blocks, grid-stride; part of the current phase)
  auto copy_rows = [&](T* dst, const T* src, int rows) {
    const long long total = (long long)rows * nc;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x)
      dst[e] = src[e];
  };
  auto too_large = [&]() {
    if (blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, AMX_ERR_TOO_LARGE);
  };
  double t = *(volatile double*)&ctl->t;
  if (taping) {
    unsigned long long* slot = produce_slot();
    phase_cfl<T, DIM>(a, a.tape + toff, slot, red);
    ++rp;
    if (!grid_sync(bar, status)) return;
  } else if (!cfl_phase()) {
    return;  // (the barrier also orders everyone's read of t before it changes)
  }
  for (long long s = 0; s < a.max_steps; ++s) {
    double dt;
    if (t >= a.t_pause) break;
    if (a.fixed_timestep) {
      dt = a.dt_fixed;
    } else {
      if (!(t < a.t_end)) break;
      dt = dt_from_maxima();
    }
    if (a.exact_end_time) dt = nanmin(dt, a.t_end - t);
    // a NaN dt is taken, as the reference takes it (its time then stops the loop)
    if (dt != dt && blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, AMX_ERR_NAN);
    const T dtT = T(dt);
    int it = 0;
    const long long idx = step0 + s;
    if (taping) {
      // one tape step (the layout above)
      if (idx + 1 > a.max_hist) { too_large(); return; }
      T* S0 = a.tape + toff;
      T* S1 = S0 + NVT * nc;
      if (!MHD) {
        T* S5 = S1 + NVG * nc;
        if (toff + (long long)(NVT + NVG + NVT) * nc > a.tape_cap) { too_large(); return; }
        if (!stage(S0, S1, nullptr, dtT, false)) return;
        if (!stage(S1, S5, S0, dtT, true)) return;
        toff = S5 - a.tape;
      } else {
        T* S2 = S1 + NVG * nc;
        T* Z0 = S2 + NVT * nc;
        // room check for the fixed rows and the iterate j (the tail S3, S4, S5 follows it)
        auto fits = [&](int j) {
          return toff + (long long)(NVT + NVG + NVT + 6 * (j + 1) + NVT + NVG + NVT) * nc <= a.tape_cap;
        };
        if (!fits(0)) { too_large(); return; }
        const T h = dtT / T(2);
        copy_rows(S2 + NVG * nc, S0 + NVG * nc, 3);
        if (!stage(S0, S1, nullptr, h, false)) return;
        if (!stage(S1, S2, S0, h, false)) return;
        // magnetic_update on S2 (_magnetic_field_update.py:37-242), iterates kept
        unsigned long long* slot = &ctl->mag[mag_pass % 3];
        if (DIM == 2) {
          const MagSrc<T, DIM> first{S2 + (DIM + 2) * nc, S2 + nc, true};
          phase_mag_iterate_direct<T, DIM>(a, S2, first, Z0, dtT, slot, red);
        } else {
          phase_mag_iterate<T, DIM>(a, S2, nullptr, Z0, dtT, slot, red, smem);
        }
        if (!grid_sync(bar, status)) return;
        double change = bits_to_double(*(volatile unsigned long long*)slot);
        if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag[(mag_pass + 2) % 3] = 0ull;
        ++mag_pass;
        int k_it = 0;
        while (change > a.tol && k_it < a.max_iters) {
          if (!fits(k_it + 1)) { too_large(); return; }
          T* cur = Z0 + 6 * (long long)k_it * nc;
          T* nxt = cur + 6 * nc;
          slot = &ctl->mag[mag_pass % 3];
          if (DIM == 2) {
            const MagSrc<T, DIM> src{cur, cur + 3 * nc, false};
            phase_mag_iterate_direct<T, DIM>(a, S2, src, nxt, dtT, slot, red);
          } else {
            phase_mag_iterate<T, DIM>(a, S2, cur, nxt, dtT, slot, red, smem);
          }
          if (!grid_sync(bar, status)) return;
          change = bits_to_double(*(volatile unsigned long long*)slot);
          if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag[(mag_pass + 2) % 3] = 0ull;
          ++mag_pass;
          ++k_it;
        }
        if (change > a.tol && blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, AMX_ERR_NOT_CONVERGED);
        if (change != change && blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, AMX_ERR_NAN);
        T* Zk = Z0 + 6 * (long long)k_it * nc;
        T* S3 = Zk + 6 * nc;
        T* S4 = S3 + NVT * nc;
        T* S5 = S4 + NVG * nc;
        unsigned long long* out = produce_slot();
        phase_mag_finalize<T, DIM>(a, S2, Zk, S3, RS == RS_LF ? out : nullptr, red);
        ++rp;
        if (!grid_sync(bar, status)) return;
        copy_rows(S5 + NVG * nc, S3 + NVG * nc, 3);
        if (!stage(S3, S4, nullptr, h, false)) return;
        if (!stage(S4, S5, S3, h, true)) return;
        toff = S5 - a.tape;
        it = k_it;
      }
    } else if (MHD) {
      if (!rk2(dtT / T(2), false)) return;
      it = magnetic(dtT);
      if (it < 0) return;
      if (!rk2(dtT / T(2), true)) return;
    } else {
      if (!rk2(dtT, true)) return;
    }
    t = t + dt;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      ctl->t = t;
      ctl->dt = dt;
      ctl->steps = step0 + s + 1;
      ctl->mag_iters = it;
      ctl->mag_iters_total += it;
      if (a.dt_hist && idx < a.max_hist) a.dt_hist[idx] = dt;
      if (a.it_hist && idx < a.max_hist) a.it_hist[idx] = it;
      if (taping) a.tape_off[idx + 1] = toff;
    }
  }
}

}  // namespace amx
