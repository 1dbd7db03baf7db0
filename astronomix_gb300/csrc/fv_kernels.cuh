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
// leave the device.  A runtime `mode` runs a single seam instead of full
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
  unsigned long long cfl[3][4];   // [slot][axis] bitwise maxima of |u_a| + c
  unsigned long long alpha[3][4]; // [slot][axis] Lax-Friedrichs alpha of a stage
  unsigned long long mag[3];      // [slot] fixed-point residual
  double dt;                      // dt of the last step taken
  double t;                       // simulation time
  long long steps;                // steps taken
  int mag_iters;                  // fixed-point iterations of the last magnetic update
  int pad0;
  long long mag_iters_total;
  unsigned int bar_count, bar_gen;
  int abort_flag;
  int status;
};

enum FVMode {
  FV_MODE_STEPS = 0,      // full time steps
  FV_MODE_CFL = 1,        // only the CFL dt (written to ctl->dt)
  FV_MODE_HYDRO_RK2 = 2,  // one RK2 update of the gas rows with dt_in * dt_scale
  FV_MODE_MAGNETIC = 3,   // one magnetic sub-step with dt_in
  FV_MODE_EVOLVE = 4,     // one _evolve_state_fv with dt_in (no CFL, no t update)
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
  int exact_end_time;
  int fixed_timestep;
  int mode;
  double dx;
  double gamma;
  double C_cfl;
  double t_end;
  double dt_fixed;   // t_end / num_timesteps (fixed mode)
  double dt_in;      // seam modes
  double dt_scale;   // seam modes
  double tol;        // fixed-point tolerance
  int max_iters;     // fixed-point cap (1000 in the reference)
  long long max_steps;
  double t_pause;    // full-step mode stops before a step that starts at t >= t_pause
};

// ---------------------------------------------------------------- tiles

template <typename T, int DIM> struct Tile;
template <typename T> struct Tile<T, 1> {
  static constexpr int T0 = 256, T1 = 1, T2 = 1;
};
template <> struct Tile<float, 2> {
  static constexpr int T0 = 8, T1 = 64, T2 = 1;
};
template <> struct Tile<double, 2> {
  static constexpr int T0 = 8, T1 = 32, T2 = 1;
};
template <> struct Tile<float, 3> {
  static constexpr int T0 = 4, T1 = 8, T2 = 32;
};
template <> struct Tile<double, 3> {
  static constexpr int T0 = 4, T1 = 4, T2 = 32;
};

constexpr int kFVThreads = 256;

template <typename T, int DIM>
struct TileGeom {
  static constexpr int NV = DIM + 2;
  static constexpr int T0 = Tile<T, DIM>::T0, T1 = Tile<T, DIM>::T1, T2 = Tile<T, DIM>::T2;
  static constexpr int H0 = T0 + 4, H1 = (DIM >= 2) ? T1 + 4 : 1, H2 = (DIM >= 3) ? T2 + 4 : 1;
  static constexpr int HALO = H0 * H1 * H2;
  static constexpr int CELLS = T0 * T1 * T2;
  static constexpr int CPT = (CELLS + kFVThreads - 1) / kFVThreads;
  static constexpr int F0 = (T0 + 1) * T1 * T2;
  static constexpr int F1 = (DIM >= 2) ? T0 * (T1 + 1) * T2 : 0;
  static constexpr int F2 = (DIM >= 3) ? T0 * T1 * (T2 + 1) : 0;
  static constexpr int FMAX = F0 > F1 ? (F0 > F2 ? F0 : F2) : (F1 > F2 ? F1 : F2);
  static constexpr size_t SMEM = sizeof(T) * (size_t)NV * (HALO + FMAX);
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
  const int n0 = (n + T0 - 1) / T0;
  const int n1 = (DIM >= 2) ? (n + T1 - 1) / T1 : 1;
  const int n2 = (DIM >= 3) ? (n + T2 - 1) / T2 : 1;
  const int t2 = (int)(tile % n2);
  const int t1 = (int)((tile / n2) % n1);
  const int t0 = (int)(tile / ((long long)n2 * n1));
  (void)n0;
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

// maps a logical (possibly out-of-domain) index onto the stored grid
template <typename T, int DIM>
__device__ __forceinline__ int map_ax(const FVArgs<T>& a, int k, int g, bool* flip) {
  const int n = a.n;
  if (g < -2) g = -2;
  if (g > n + 1) g = n + 1;
  if (a.periodic_roll) return wrap(g, n);
  return map_index(g, n, a.bc[k], DIM == 1, flip);
}

// ------------------------------------------------------------ CFL phase

// Per-axis maxima of |u_a| + c over all cells (the ghost cells of the
// reference are copies of interior cells and add nothing to the maximum).
template <typename T, int DIM>
__device__ __noinline__ void phase_cfl(const FVArgs<T>& a, unsigned long long* slot, double* red) {
  const T gamma = T(a.gamma);
  T m[3] = {T(0), T(0), T(0)};
  const long long nc = a.ncells;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (long long)gridDim.x * blockDim.x) {
    const T rho = a.state[c];
    const T p = a.state[(DIM + 1) * nc + c];
    const T cs = sound_speed(rho, p, gamma);
#pragma unroll
    for (int k = 0; k < DIM; ++k) m[k] = nanmax(m[k], Num<T>::abs_(a.state[(1 + k) * nc + c]) + cs);
  }
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    const double r = block_max<double>((double)m[k], red);
    if (threadIdx.x == 0) atomic_max_nonneg(&slot[k], r);
  }
}

// Lax-Friedrichs alpha of a stage input (max over cells of |u_d| + c).
template <typename T, int DIM>
__device__ __noinline__ void phase_alpha(const FVArgs<T>& a, const T* P, unsigned long long* slot, double* red) {
  const T gamma = T(a.gamma);
  T m[3] = {T(0), T(0), T(0)};
  const long long nc = a.ncells;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (long long)gridDim.x * blockDim.x) {
    const T cs = sound_speed(P[c], P[(DIM + 1) * nc + c], gamma);
#pragma unroll
    for (int k = 0; k < DIM; ++k) m[k] = nanmax(m[k], Num<T>::abs_(P[(1 + k) * nc + c]) + cs);
  }
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    const double r = block_max<double>((double)m[k], red);
    if (threadIdx.x == 0) atomic_max_nonneg(&slot[k], r);
  }
}

// ------------------------------------------------------------ hydro stage

// One _evolve_gas_state_unsplit_inner (evolve_state.py:339-414):
//   U = cons(P_in); for each axis: U += (1/dx) (F[i-1/2] - F[i+1/2]) dt;
//   P_out = prim(U)
// and, when `P0` is given, the RK2 combination of evolve_state.py:456-469:
//   P_out = prim(0.5 (cons(P0) + cons(prim(U)))).
// `alpha` holds the Lax-Friedrichs alpha per axis (unused otherwise).
template <typename T, int DIM, int RS>
__device__ __noinline__ void phase_hydro_stage(const FVArgs<T>& a, const T* __restrict__ Pin, T* Pout,
                                  const T* P0, T dt, const T* alpha, T* smem) {
  using G = TileGeom<T, DIM>;
  constexpr int NV = G::NV;
  const int n = a.n;
  const long long nc = a.ncells;
  const T gamma = T(a.gamma);
  const T dxT = T(a.dx);
  const T inv_dx = T(1.0 / a.dx);
  T* sP = smem;                      // [NV][HALO]
  T* sF = smem + NV * G::HALO;       // [NV][FMAX]
  const long long ntiles = fv_num_tiles<DIM>(n, G::T0, G::T1, G::T2);

  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int o[3];
    tile_origin<DIM>(tile, n, G::T0, G::T1, G::T2, o);

    // ---- load the halo'd tile of primitives (boundary-mapped)
    for (int e = threadIdx.x; e < G::HALO; e += blockDim.x) {
      const int h2 = e % G::H2;
      const int h1 = (e / G::H2) % G::H1;
      const int h0 = e / (G::H2 * G::H1);
      bool f0 = false, f1 = false, f2 = false;
      const int i0 = map_ax<T, DIM>(a, 0, o[0] + h0 - 2, &f0);
      const int i1 = (DIM >= 2) ? map_ax<T, DIM>(a, 1, o[1] + h1 - 2, &f1) : 0;
      const int i2 = (DIM >= 3) ? map_ax<T, DIM>(a, 2, o[2] + h2 - 2, &f2) : 0;
      const long long c = cell_index<DIM>(i0, i1, i2, n);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        T val = Pin[v * nc + c];
        if ((v == 1 && f0) || (v == 2 && f1) || (v == 3 && f2)) val = -val;
        sP[v * G::HALO + e] = val;
      }
    }
    __syncthreads();

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

    // ---- axes in the reference order x, y, z
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const int E0 = G::T0 + (k == 0), E1 = (DIM >= 2) ? G::T1 + (k == 1) : 1, E2 = (DIM >= 3) ? G::T2 + (k == 2) : 1;
      const int nf = E0 * E1 * E2;
      const int stride = (k == 0) ? G::H1 * G::H2 : ((k == 1) ? G::H2 : 1);
      for (int f = threadIdx.x; f < nf; f += blockDim.x) {
        const int f2 = f % E2, f1 = (f / E2) % E1, f0 = f / (E2 * E1);
        // halo index of the cell right of the face (local cell c = face index)
        const int h = ((f0 + 2) * G::H1 + (DIM >= 2 ? f1 + 2 : 0)) * G::H2 + (DIM >= 3 ? f2 + 2 : 0);
        T qL[NV], qR[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const T* s = sP + v * G::HALO + h;
          const T qm2 = s[-2 * stride], qm1 = s[-stride], q0 = s[0], qp1 = s[stride];
          const T gm1 = limited((qm1 - qm2) / dxT, (q0 - qm1) / dxT, a.limiter, dxT);
          const T g0 = limited((q0 - qm1) / dxT, (qp1 - q0) / dxT, a.limiter, dxT);
          qL[v] = qm1 + gm1 * dxT / T(2);
          qR[v] = q0 - g0 * dxT / T(2);
        }
        T F[NV];
        riemann<T, DIM, RS>(qL, qR, k + 1, gamma, alpha ? alpha[k] : T(0), a.lm != 0, F);
        // face f stored at its own (E0,E1,E2) index
#pragma unroll
        for (int v = 0; v < NV; ++v) sF[v * G::FMAX + f] = F[v];
      }
      __syncthreads();
#pragma unroll
      for (int j = 0; j < G::CPT; ++j) {
        const int cl = threadIdx.x + j * kFVThreads;
        if (cl < G::CELLS) {
          const int c2 = cl % G::T2, c1 = (cl / G::T2) % G::T1, c0 = cl / (G::T2 * G::T1);
          const int fl = (c0 * E1 + c1) * E2 + c2;  // face i-1/2 of the cell
          const int fr = fl + ((k == 0) ? E1 * E2 : ((k == 1) ? E2 : 1));
#pragma unroll
          for (int v = 0; v < NV; ++v)
            U[j][v] = U[j][v] + inv_dx * (sF[v * G::FMAX + fl] - sF[v * G::FMAX + fr]) * dt;
        }
      }
      __syncthreads();
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
        }
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ magnetic sub-step

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

template <typename T>
__device__ __forceinline__ void cross3(const T* a, const T* b, T* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

template <typename T, int DIM>
__device__ __forceinline__ long long mag_neighbor(const FVArgs<T>& a, const int* ic, int k, int off) {
  int j[3] = {ic[0], ic[1], ic[2]};
  bool flip = false;
  j[k] = map_ax<T, DIM>(a, k, ic[k] + off, &flip);
  return cell_index<DIM>(j[0], j[1], j[2], a.n);
}

// One evaluation of the fixed-point map (_magnetic_field_update.py:82-105,
// :143-165): writes B_{k+1}, v_{k+1} to `dst` and folds max |B_k - B_{k+1}|,
// max |v_k - v_{k+1}| into `slot`.
template <typename T, int DIM>
__device__ __noinline__ void phase_mag_iterate(const FVArgs<T>& a, MagSrc<T, DIM> src, T* dst, T dt,
                                  unsigned long long* slot, double* red) {
  const long long nc = a.ncells;
  const int n = a.n;
  const T dx = T(a.dx);
  const MagSrc<T, DIM> s0{a.state + (DIM + 2) * nc, a.state + nc, true};  // B0, v0
  const T* rho = a.state;
  const bool midpoint = (a.integrator == 0);
  T change = T(0);
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (long long)gridDim.x * blockDim.x) {
    int ic[3];
    if (DIM == 2) { ic[0] = (int)(c / n); ic[1] = (int)(c % n); ic[2] = 0; }
    else { ic[2] = (int)(c % n); ic[1] = (int)((c / n) % n); ic[0] = (int)(c / ((long long)n * n)); }
    // averaged fields at the cell and its 2*DIM neighbours
    T Bc[3], vc[3], B0c[3], v0c[3];
    auto avg_at = [&](long long cc, T* Ba, T* va, T* Bk_out, T* vk_out, T* B0_out, T* v0_out) {
      T Bk[3], vk[3], B0[3], v0[3];
      load_Bv<T, DIM>(src, cc, nc, Bk, vk);
      load_Bv<T, DIM>(s0, cc, nc, B0, v0);
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
      avg_at(mag_neighbor<T, DIM>(a, ic, k, +1), Ba, va, nullptr, nullptr, nullptr, nullptr);
      cross3(Ba, va, Ep[k]);
#pragma unroll
      for (int i = 0; i < 3; ++i) Bp[k][i] = Ba[i];
      avg_at(mag_neighbor<T, DIM>(a, ic, k, -1), Ba, va, nullptr, nullptr, nullptr, nullptr);
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
  const double r = block_max<double>((double)change, red);
  if (threadIdx.x == 0) atomic_max_nonneg(slot, r);
}

// Pressure refresh with gamma = 5/3 and write-back (_magnetic_field_update.py:208-242).
template <typename T, int DIM>
__device__ __noinline__ void phase_mag_finalize(const FVArgs<T>& a, const T* Bv) {
  const long long nc = a.ncells;
  const T g53 = T(5.0 / 3.0);
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (long long)gridDim.x * blockDim.x) {
    const T rho = a.state[c];
    const T p = a.state[(DIM + 1) * nc + c];
    T v0[3];
    v0[0] = a.state[nc + c];
    v0[1] = a.state[2 * nc + c];
    v0[2] = (DIM == 3) ? a.state[3 * nc + c] : T(0);
    T vn[3], Bn[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) { Bn[i] = Bv[i * nc + c]; vn[i] = Bv[(3 + i) * nc + c]; }
    const T v0abs = Num<T>::sqrt_(v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
    const T vnabs = Num<T>::sqrt_(vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2]);
    T E = total_energy(rho, v0abs, p, g53);
    E = E - T(0.5) * rho * (v0abs * v0abs) + T(0.5) * rho * (vnabs * vnabs);
    const T pn = pressure_from_energy(E, rho, vnabs, g53);
#pragma unroll
    for (int i = 0; i < DIM; ++i) a.state[(1 + i) * nc + c] = vn[i];
    a.state[(DIM + 1) * nc + c] = pn;
#pragma unroll
    for (int i = 0; i < 3; ++i) a.state[(DIM + 2 + i) * nc + c] = Bn[i];
  }
}

// ------------------------------------------------------------ the kernel

template <typename T, int DIM, int RS, bool MHD>
__global__ void __launch_bounds__(kFVThreads)
fv_run_kernel(FVArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  __shared__ double red[32];
  FVControl* ctl = a.ctl;
  int* status = &ctl->status;
  const GridBarrier bar{&ctl->bar_count, &ctl->bar_gen, &ctl->abort_flag};
  const long long nc = a.ncells;
  T* gas = a.state;
  __shared__ T s_alpha[3];

  int cfl_pass = 0, mag_pass = 0, lf_pass = 0;

  // LF alpha of a stage input; returns false on a barrier failure
  auto stage_alpha = [&](const T* P) -> bool {
    if (RS != RS_LF) return true;
    unsigned long long* slot = ctl->alpha[lf_pass % 3];
    phase_alpha<T, DIM>(a, P, slot, red);
    if (!grid_sync(bar, status)) return false;
    if (threadIdx.x < DIM) s_alpha[threadIdx.x] = T(bits_to_double(slot[threadIdx.x]));
    if (blockIdx.x == 0 && threadIdx.x < 4) ctl->alpha[(lf_pass + 2) % 3][threadIdx.x] = 0ull;
    __syncthreads();
    ++lf_pass;
    return true;
  };

  // one RK2 update of the gas rows with stage dt `h` (evolve_state.py:419-488)
  auto rk2 = [&](T h) -> bool {
    if (!stage_alpha(gas)) return false;
    phase_hydro_stage<T, DIM, RS>(a, gas, a.p1, nullptr, h, RS == RS_LF ? s_alpha : nullptr, smem);
    if (!grid_sync(bar, status)) return false;
    if (!stage_alpha(a.p1)) return false;
    phase_hydro_stage<T, DIM, RS>(a, a.p1, gas, gas, h, RS == RS_LF ? s_alpha : nullptr, smem);
    return grid_sync(bar, status);
  };

  // magnetic_update (_magnetic_field_update.py:37-242); returns iterations or -1
  auto magnetic = [&](T h) -> int {
    const MagSrc<T, DIM> first{gas + (DIM + 2) * nc, gas + nc, true};
    unsigned long long* slot = &ctl->mag[mag_pass % 3];
    phase_mag_iterate<T, DIM>(a, first, a.mag0, h, slot, red);
    if (!grid_sync(bar, status)) return -1;
    double change = bits_to_double(*(volatile unsigned long long*)slot);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag[(mag_pass + 2) % 3] = 0ull;
    ++mag_pass;
    int it = 0;
    T* cur = a.mag0;
    T* nxt = a.mag1;
    while (change > a.tol && it < a.max_iters) {
      const MagSrc<T, DIM> src{cur, cur + 3 * nc, false};
      slot = &ctl->mag[mag_pass % 3];
      phase_mag_iterate<T, DIM>(a, src, nxt, h, slot, red);
      if (!grid_sync(bar, status)) return -1;
      change = bits_to_double(*(volatile unsigned long long*)slot);
      if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag[(mag_pass + 2) % 3] = 0ull;
      ++mag_pass;
      ++it;
      T* tmp = cur; cur = nxt; nxt = tmp;
    }
    if (change > a.tol && blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, AMX_ERR_NOT_CONVERGED);
    if (change != change && blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, AMX_ERR_NAN);
    phase_mag_finalize<T, DIM>(a, cur);
    if (!grid_sync(bar, status)) return -1;
    return it;
  };

  auto cfl = [&](double* dt_out) -> bool {
    unsigned long long* slot = ctl->cfl[cfl_pass % 3];
    phase_cfl<T, DIM>(a, slot, red);
    if (!grid_sync(bar, status)) return false;
    double sum = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const double m = bits_to_double(*(volatile unsigned long long*)&slot[k]);
      sum = (k == 0) ? m / a.dx : sum + m / a.dx;
    }
    *dt_out = a.C_cfl * 1.0 / sum;
    if (blockIdx.x == 0 && threadIdx.x < 4) ctl->cfl[(cfl_pass + 2) % 3][threadIdx.x] = 0ull;
    ++cfl_pass;
    return true;
  };

  if (a.mode == FV_MODE_CFL) {
    double dt;
    if (!cfl(&dt)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->dt = dt;
    return;
  }
  if (a.mode == FV_MODE_HYDRO_RK2) {
    rk2(T(a.dt_in * a.dt_scale));
    return;
  }
  if (a.mode == FV_MODE_MAGNETIC) {
    if (!MHD) return;
    const int it = magnetic(T(a.dt_in));
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag_iters = it;
    return;
  }
  if (a.mode == FV_MODE_EVOLVE) {
    const T dtT = T(a.dt_in);
    if (MHD) {
      if (!rk2(dtT / T(2))) return;
      const int it = magnetic(dtT);
      if (it < 0) return;
      if (blockIdx.x == 0 && threadIdx.x == 0) ctl->mag_iters = it;
      rk2(dtT / T(2));
    } else {
      rk2(dtT);
    }
    return;
  }

  // ---- full time steps (time_integration.py:386-762)
  const long long step0 = *(volatile long long*)&ctl->steps;
  double t = *(volatile double*)&ctl->t;
  if (!grid_sync(bar, status)) return;  // everyone has read t before it changes
  for (long long s = 0; s < a.max_steps; ++s) {
    double dt;
    if (t >= a.t_pause) break;
    if (a.fixed_timestep) {
      dt = a.dt_fixed;
    } else {
      if (!(t < a.t_end)) break;
      if (!cfl(&dt)) return;
    }
    if (a.exact_end_time) dt = fmin(dt, a.t_end - t);
    const T dtT = T(dt);
    int it = 0;
    if (MHD) {
      if (!rk2(dtT / T(2))) return;
      it = magnetic(dtT);
      if (it < 0) return;
      if (!rk2(dtT / T(2))) return;
    } else {
      if (!rk2(dtT)) return;
    }
    t = t + dt;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      ctl->t = t;
      ctl->dt = dt;
      ctl->steps = step0 + s + 1;
      ctl->mag_iters = it;
      ctl->mag_iters_total += it;
      const long long idx = step0 + s;
      if (a.dt_hist && idx < a.max_hist) a.dt_hist[idx] = dt;
      if (a.it_hist && idx < a.max_hist) a.it_hist[idx] = it;
    }
  }
}

}  // namespace amx
