// Self-gravity of the finite-volume scheme: the FFT Poisson solve (cuFFT
// transforms, own pack / Green's function / crop kernels) and the
// gravitational source term applied after every gas update.
//
// References (astronomix 0.5.1):
//   _physics_modules/_self_gravity/_poisson_solver.py:17-151  the potential
//   _physics_modules/_self_gravity/_self_gravity.py:68-337    source term per axis
//   _physics_modules/_self_gravity/_self_gravity.py:341-390   _apply_self_gravity
//
// The reference solves on the array it holds: with ghost-cell handling the
// padded grid (n + 4 cells per axis, ghost cells filled by the boundary
// handler), with periodic roll the stored grid.  This code solves on the
// same grid, filling the padded cells by index mapping, so that the
// potential (and every acceleration) equals the reference's.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <new>

#include "../../include/amx.h"
#include "amx_common.cuh"
#include "fv_kernels.cuh"
#include "gravity.h"

namespace amx {

namespace {

constexpr int kGThreads = 256;
constexpr int kSumBlocks = 304;

// How the FFT grid maps onto the stored cells.
struct GravGrid {
  int dim;
  int n;     // stored cells per axis
  int goff;  // 2 with ghost-cell handling (the padded grid), 0 otherwise
  int M;     // n + 2 goff: the grid the reference solves on
  int E;     // FFT extent per axis: M (periodic) or 2 M (open, zero padded)
  int roll;  // periodic roll handling: stencil offsets wrap
  AxisBC bc[3];
};

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = cufftComplex; };
template <> struct Cplx<double> { using type = cufftDoubleComplex; };

__host__ __device__ inline long long ipow_ll(long long b, int e) {
  long long r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

// stored cell of the padded-grid cell (p0, p1, p2) (no velocity flip: density only)
__device__ __forceinline__ long long stored_cell(const GravGrid& g, int p0, int p1, int p2) {
  bool f = false;
  const int i0 = map_index(p0 - g.goff, g.n, g.bc[0], g.dim == 1, &f);
  const int i1 = g.dim >= 2 ? map_index(p1 - g.goff, g.n, g.bc[1], false, &f) : 0;
  const int i2 = g.dim >= 3 ? map_index(p2 - g.goff, g.n, g.bc[2], false, &f) : 0;
  if (g.dim == 1) return i0;
  if (g.dim == 2) return (long long)i0 * g.n + i1;
  return ((long long)i0 * g.n + i1) * g.n + i2;
}

__device__ __forceinline__ void split_coords(long long e, int ext, int dim, int* p) {
  p[0] = p[1] = p[2] = 0;
  for (int k = dim - 1; k >= 0; --k) {
    p[k] = (int)(e % ext);
    e /= ext;
  }
}

__device__ __forceinline__ long long ext_index(const GravGrid& g, const int* p) {
  long long r = p[0];
  for (int k = 1; k < g.dim; ++k) r = r * g.E + p[k];
  return r;
}

__device__ __forceinline__ double block_sum(double v, double* scratch) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int w = 0; w < nw; ++w) r += scratch[w];
  }
  return r;  // valid in thread 0
}

// Mean of the density over the solve grid (periodic only; _poisson_solver.py:82-84).
// Deterministic: per-block partial sums, added in block order by the last block.
template <typename T>
__global__ void __launch_bounds__(kGThreads) k_density_mean(const T* __restrict__ rho, GravGrid g,
                                                            double* partial, unsigned int* counter, double* mean,
                                                            const int* active) {
  __shared__ double scratch[32];
  __shared__ bool last;
  if (active && !*(volatile const int*)active) return;
  const long long total = ipow_ll(g.M, g.dim);
  double s = 0.0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int p[3];
    split_coords(e, g.M, g.dim, p);
    s += (double)rho[stored_cell(g, p[0], p[1], p[2])];
  }
  s = block_sum(s, scratch);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double tot = 0.0;
    for (unsigned int b = 0; b < gridDim.x; ++b) tot += ((volatile double*)partial)[b];
    *mean = tot / (double)total;
    *counter = 0u;
  }
}

// The density on the solve grid (minus its mean when periodic) into the
// corner of the FFT input; the rest of an open-boundary input stays zero.
template <typename T>
__global__ void __launch_bounds__(kGThreads) k_density_pack(const T* __restrict__ rho, GravGrid g,
                                                            const double* mean, T* __restrict__ fin,
                                                            const int* active) {
  if (active && !*(volatile const int*)active) return;
  const long long total = ipow_ll(g.M, g.dim);
  const T mu = mean ? T(*mean) : T(0);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int p[3];
    split_coords(e, g.M, g.dim, p);
    const T r = rho[stored_cell(g, p[0], p[1], p[2])];
    fin[ext_index(g, p)] = mean ? r - mu : r;
  }
}

// Periodic Green's function (_poisson_solver.py:86-113) on the half spectrum,
// times `scale` (the inverse transform's 1 / E^d): the wave numbers are
// 2 pi fftfreq(E, dx), -4 pi G / k^2 and -1 / (4 pi) at k = 0.
template <typename C>
__global__ void __launch_bounds__(kGThreads) k_green_periodic(C* spec, GravGrid g, double dx, double G, double scale,
                                                              const int* active) {
  if (active && !*(volatile const int*)active) return;
  const int E = g.E, H = E / 2 + 1;
  const long long total = ipow_ll(E, g.dim - 1) * H;
  const double val = 1.0 / ((double)E * dx);
  const double pi = 3.141592653589793;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    // wave-number indices of the half spectrum (last axis: 0 .. E/2)
    int js[3] = {0, 0, 0};
    long long rest = e;
    for (int k = g.dim - 1; k >= 0; --k) {
      const int ext = (k == g.dim - 1) ? H : E;
      const int j = (int)(rest % ext);
      rest /= ext;
      js[k] = (j <= (E - 1) / 2) ? j : j - E;
    }
    // k_x^2 + k_y^2 + k_z^2 in axis order, k = fftfreq(E, dx) * 2 * pi
    double k2 = 0.0;
    for (int k = 0; k < g.dim; ++k) {
      const double kk = (double)js[k] * val * 2.0 * pi;
      k2 = (k == 0) ? kk * kk : k2 + kk * kk;
    }
    if (k2 == 0.0) k2 = 1e-12;
    const double green = (k2 > 1e-12) ? (-4.0 * pi * G) / k2 : -1.0 / (4.0 * pi);
    const double f = green * scale;
    C z = spec[e];
    z.x = z.x * f;
    z.y = z.y * f;
    spec[e] = z;
  }
}

// Open boundaries: the spectrum times the isolated kernel's spectrum (G = 1),
// times G and `scale` (dx^d / E^d).
template <typename C>
__global__ void __launch_bounds__(kGThreads) k_green_open(C* spec, const C* __restrict__ kspec, long long total,
                                                          double f, const int* active) {
  if (active && !*(volatile const int*)active) return;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const C a = spec[e], b = kspec[e];
    C z;
    z.x = (a.x * b.x - a.y * b.y) * f;
    z.y = (a.x * b.y + a.y * b.x) * f;
    spec[e] = z;
  }
}

// The isolated kernel of _poisson_solver.py:115-147 with G = 1 on the padded
// FFT grid: minimum-image distances, r = 0 replaced by dx; -2 pi r (1D),
// -2 log r (2D), -1 / r (3D).
__global__ void __launch_bounds__(kGThreads) k_open_kernel(double* out, GravGrid g, double dx) {
  const long long total = ipow_ll(g.E, g.dim);
  const double pi = 3.141592653589793;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int p[3];
    split_coords(e, g.E, g.dim, p);
    double x[3];
    for (int k = 0; k < 3; ++k) {
      const int j = p[k] < g.M ? p[k] : g.E - p[k];
      x[k] = (double)j * dx;
    }
    double r;
    if (g.dim == 1) r = x[0];
    else if (g.dim == 2) r = sqrt(x[0] * x[0] + x[1] * x[1]);
    else r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    const double rs = (r == 0.0) ? dx : r;
    double v;
    if (g.dim == 1) v = -2.0 * pi * r;
    else if (g.dim == 2) v = -2.0 * log(rs);
    else v = -1.0 / rs;
    out[e] = v;
  }
}

template <typename C, typename D>
__global__ void k_convert_spectrum(const D* in, C* out, long long total) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    C z;
    z.x = in[e].x;
    z.y = in[e].y;
    out[e] = z;
  }
}

// The solve grid's corner of the inverse transform into a dense n^d array.
template <typename T>
__global__ void k_crop(const T* __restrict__ fout, GravGrid g, T* __restrict__ out) {
  const long long total = ipow_ll(g.M, g.dim);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int p[3];
    split_coords(e, g.M, g.dim, p);
    out[e] = fout[ext_index(g, p)];
  }
}

// ----------------------------------------------------------- source term

template <typename T>
struct GravSrc {
  const T* old;    // gas rows before the gas update
  T* state;        // gas rows after it (updated in place)
  const T* phi;    // potential on the FFT grid (solve-grid corner)
  GravGrid g;
  long long nc;
  const FVControl* ctl;
  double dt_scale;
  double dx;
  double gamma;
  int version;
  int lm;
  int split;
  int first_order;
  int limiter;
};

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

// _gravitational_source_term_along_axis for every axis and the explicit
// update of _apply_self_gravity, one cell per thread: the central
// acceleration -(phi[i+1] - phi[i-1]) / 2dx gives the momentum source rho a;
// the energy source is rho v a (SIMPLE_SOURCE_TERM) or the mass fluxes
// through the cell's two interfaces, from the interface states of the old
// state and the configured Riemann solver, times the one-sided
// accelerations, shared per version.  U += dt S, back to primitives.
template <typename T, int DIM, int RS>
__global__ void __launch_bounds__(kGThreads) k_grav_source(GravSrc<T> a) {
  constexpr int NV = DIM + 2, P = DIM + 1;
  const FVControl* ctl = a.ctl;
  if (!*(volatile const int*)&ctl->active) return;
  const T h = T(*(volatile const double*)&ctl->dt * a.dt_scale);
  const T gamma = T(a.gamma);
  const T dxT = T(a.dx);
  const T two_dx = T(2.0 * a.dx);
  const GravGrid g = a.g;
  const int n = g.n;
  const long long nc = a.nc;
  const int version = a.version;
  const bool lm = a.lm != 0;
  T alpha[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) alpha[k] = T(((volatile const double*)ctl->seam_maxima)[k]);
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
    int ic[3] = {0, 0, 0};
    {
      long long r = c;
      for (int k = DIM - 1; k >= 0; --k) {
        ic[k] = (int)(r % n);
        r /= n;
      }
    }
    T q0[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) q0[v] = a.old[v * nc + c];
    const T rho = q0[0];
    T mS[DIM];
    T eS = T(0);
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      // potential at i-1, i, i+1 along k
      int p[3] = {ic[0] + g.goff, ic[1] + g.goff, ic[2] + g.goff};
      T ph[3];
#pragma unroll
      for (int o = -1; o <= 1; ++o) {
        int pp[3] = {p[0], p[1], p[2]};
        pp[k] = g.roll ? wrap(p[k] + o, n) : p[k] + o;
        ph[o + 1] = a.phi[ext_index(g, pp)];
      }
      const T acc = -(ph[2] - ph[0]) / two_dx;
      mS[k] = rho * acc;
      T e;
      if (version == AMX_SIMPLE_SOURCE_TERM) {
        e = rho * q0[k + 1] * acc;
      } else {
        // the old state at i-2 .. i+2 along k (boundary mapped)
        T q[5][NV];
#pragma unroll
        for (int o = -2; o <= 2; ++o) {
          if (o == 0) {
#pragma unroll
            for (int v = 0; v < NV; ++v) q[2][v] = q0[v];
            continue;
          }
          int jc[3] = {ic[0], ic[1], ic[2]};
          bool flip = false;
          jc[k] = g.roll ? wrap(ic[k] + o, n) : map_index(ic[k] + o, n, g.bc[k], DIM == 1, &flip);
          long long cc = jc[0];
          if (DIM >= 2) cc = cc * n + jc[1];
          if (DIM >= 3) cc = cc * n + jc[2];
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            T val = a.old[v * nc + cc];
            if (flip && v == k + 1) val = -val;
            q[o + 2][v] = val;
          }
        }
        // interface states of the faces i-1/2 (a) and i+1/2 (b)
        T aL[NV], aR[NV], bL[NV], bR[NV];
        if (a.first_order) {
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            aL[v] = q[1][v];
            aR[v] = q[2][v];
            bL[v] = q[2][v];
            bR[v] = q[3][v];
          }
        } else if (a.split) {
          T lo[NV], hi[NV];
          muscl_states<T, DIM>(q[0], q[1], q[2], k + 1, gamma, h, dxT, a.limiter, lo, hi);
#pragma unroll
          for (int v = 0; v < NV; ++v) aL[v] = hi[v];
          muscl_states<T, DIM>(q[1], q[2], q[3], k + 1, gamma, h, dxT, a.limiter, lo, hi);
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            aR[v] = lo[v];
            bL[v] = hi[v];
          }
          muscl_states<T, DIM>(q[2], q[3], q[4], k + 1, gamma, h, dxT, a.limiter, lo, hi);
#pragma unroll
          for (int v = 0; v < NV; ++v) bR[v] = lo[v];
        } else {
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            const T dm = limited((q[1][v] - q[0][v]) / dxT, (q[2][v] - q[1][v]) / dxT, a.limiter, dxT) * dxT / T(2);
            const T d0 = limited((q[2][v] - q[1][v]) / dxT, (q[3][v] - q[2][v]) / dxT, a.limiter, dxT) * dxT / T(2);
            const T dp = limited((q[3][v] - q[2][v]) / dxT, (q[4][v] - q[3][v]) / dxT, a.limiter, dxT) * dxT / T(2);
            aL[v] = q[1][v] + dm;
            aR[v] = q[2][v] - d0;
            bL[v] = q[2][v] + d0;
            bR[v] = q[3][v] - dp;
          }
        }
        T f_to_im1, f_to_ip1;
        if (version == AMX_RIEMANN_SPLIT || version == AMX_RIEMANN_SPLIT_UNSTABLE) {
          const bool unstable = version == AMX_RIEMANN_SPLIT_UNSTABLE;
          T x, y;
          riemann_split_mass<T, DIM>(aL, aR, k + 1, gamma, lm, unstable, &f_to_im1, &x);
          riemann_split_mass<T, DIM>(bL, bR, k + 1, gamma, lm, unstable, &y, &f_to_ip1);
        } else {
          T Fa[NV], Fb[NV];
          riemann<T, DIM, RS>(aL, aR, k + 1, gamma, alpha[k], lm, Fa);
          riemann<T, DIM, RS>(bL, bR, k + 1, gamma, alpha[k], lm, Fb);
          if (version == AMX_DONOR_ACCOUNTING) {
            f_to_ip1 = jmax(Fb[0], T(0));
            f_to_im1 = jmin(Fa[0], T(0));
          } else {  // HALF_SPLIT
            f_to_ip1 = T(0.5) * Fb[0];
            f_to_im1 = T(0.5) * Fa[0];
          }
        }
        const T acc_b = -(ph[1] - ph[0]) / dxT;
        const T acc_f = -(ph[2] - ph[1]) / dxT;
        e = f_to_im1 * acc_b + f_to_ip1 * acc_f;
      }
      eS = (k == 0) ? e : eS + e;
    }
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

__global__ void k_grav_advance(FVControl* ctl, double* dt_hist, int* it_hist, long long max_hist, int mhd) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (!ctl->active) return;
  const double dt = ctl->dt;
  ctl->t = ctl->t + dt;
  const long long idx = ctl->steps;
  ctl->steps = idx + 1;
  const int it = mhd ? ctl->mag_iters : 0;
  ctl->mag_iters_total += it;
  if (dt_hist && idx < max_hist) dt_hist[idx] = dt;
  if (it_hist && idx < max_hist) it_hist[idx] = it;
}

inline int cuda_ok(cudaError_t e) { return e == cudaSuccess ? AMX_OK : AMX_ERR_CUDA; }
inline int fft_ok(cufftResult r) { return r == CUFFT_SUCCESS ? AMX_OK : AMX_ERR_CUDA; }
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int grid_for(long long work, int num_sms) {
  const long long b = (work + kGThreads - 1) / kGThreads;
  const long long cap = (long long)num_sms * 8;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

}  // namespace

struct GravPlan {
  GravGrid g{};
  int dtype = AMX_F32;
  bool periodic = true;
  double dx = 1.0;
  int version = AMX_DONOR_ACCOUNTING;
  int rs = AMX_HLL;
  int lm = 0, split = 0, first_order = 0, limiter = AMX_MINMOD;
  long long ncells = 0;
  int num_sms = 1;
  cufftHandle fwd = 0, inv = 0;
  bool have_fwd = false, have_inv = false;
  unsigned char* mem = nullptr;
  size_t bytes = 0;
  void* fin = nullptr;    // FFT input (E^d real)
  void* fout = nullptr;   // inverse transform (E^d real): the potential in its solve-grid corner
  void* spec = nullptr;   // half spectrum
  void* kspec = nullptr;  // open: the isolated kernel's half spectrum
  void* old = nullptr;    // run: gas rows of the state before a gas update
  double* partial = nullptr;
  unsigned int* counter = nullptr;
  double* mean = nullptr;
};

namespace {

// Allocates the solver of a grid; `old_rows` gas rows of scratch for runs.
int solver_create(const GravGrid& g, double dx, bool periodic, int dtype, int old_rows, long long ncells,
                  GravPlan** out) {
  GravPlan* p = new (std::nothrow) GravPlan();
  if (!p) return AMX_ERR_INVALID_ARG;
  p->g = g;
  p->dx = dx;
  p->periodic = periodic;
  p->dtype = dtype;
  p->ncells = ncells;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t elem = dtype == AMX_F32 ? 4 : 8;
  const long long nreal = ipow_ll(g.E, g.dim);
  const long long ncplx = ipow_ll(g.E, g.dim - 1) * (g.E / 2 + 1);
  size_t off = 0;
  const size_t o_in = off; off = align256(off + elem * nreal);
  const size_t o_out = off; off = align256(off + elem * nreal);
  const size_t o_sp = off; off = align256(off + 2 * elem * ncplx);
  const size_t o_ks = off; off = align256(off + (periodic ? 0 : 2 * elem * ncplx));
  const size_t o_old = off; off = align256(off + elem * (size_t)old_rows * ncells);
  const size_t o_part = off; off = align256(off + sizeof(double) * kSumBlocks);
  const size_t o_cnt = off; off = align256(off + sizeof(unsigned int));
  const size_t o_mean = off; off = align256(off + sizeof(double));
  p->bytes = off;
  if (cudaMalloc(&p->mem, off) != cudaSuccess) { delete p; return AMX_ERR_CUDA; }
  cudaMemset(p->mem, 0, off);
  p->fin = p->mem + o_in;
  p->fout = p->mem + o_out;
  p->spec = p->mem + o_sp;
  p->kspec = periodic ? nullptr : p->mem + o_ks;
  p->old = old_rows ? p->mem + o_old : nullptr;
  p->partial = reinterpret_cast<double*>(p->mem + o_part);
  p->counter = reinterpret_cast<unsigned int*>(p->mem + o_cnt);
  p->mean = reinterpret_cast<double*>(p->mem + o_mean);
  int nn[3] = {g.E, g.E, g.E};
  int rc = fft_ok(cufftPlanMany(&p->fwd, g.dim, nn, nullptr, 1, 0, nullptr, 1, 0,
                                dtype == AMX_F32 ? CUFFT_R2C : CUFFT_D2Z, 1));
  p->have_fwd = rc == AMX_OK;
  if (!rc) {
    rc = fft_ok(cufftPlanMany(&p->inv, g.dim, nn, nullptr, 1, 0, nullptr, 1, 0,
                              dtype == AMX_F32 ? CUFFT_C2R : CUFFT_Z2D, 1));
    p->have_inv = rc == AMX_OK;
  }
  if (!rc && !periodic) {
    // the isolated kernel's spectrum, in FP64 whatever the state precision
    double* kr = nullptr;
    cufftDoubleComplex* kc = nullptr;
    cufftHandle kp = 0;
    rc = cuda_ok(cudaMalloc(&kr, sizeof(double) * nreal));
    if (!rc) rc = cuda_ok(cudaMalloc(&kc, sizeof(cufftDoubleComplex) * ncplx));
    if (!rc) rc = fft_ok(cufftPlanMany(&kp, g.dim, nn, nullptr, 1, 0, nullptr, 1, 0, CUFFT_D2Z, 1));
    if (!rc) {
      k_open_kernel<<<grid_for(nreal, p->num_sms), kGThreads>>>(kr, g, dx);
      rc = fft_ok(cufftExecD2Z(kp, kr, kc));
      if (!rc) {
        if (dtype == AMX_F32)
          k_convert_spectrum<cufftComplex, cufftDoubleComplex>
              <<<grid_for(ncplx, p->num_sms), kGThreads>>>(kc, static_cast<cufftComplex*>(p->kspec), ncplx);
        else
          rc = cuda_ok(cudaMemcpy(p->kspec, kc, sizeof(cufftDoubleComplex) * ncplx, cudaMemcpyDeviceToDevice));
      }
      rc |= cuda_ok(cudaDeviceSynchronize());
      cufftDestroy(kp);
    }
    if (kr) cudaFree(kr);
    if (kc) cudaFree(kc);
  }
  rc |= cuda_ok(cudaDeviceSynchronize());
  if (rc) {
    grav_plan_destroy(p);
    return rc ? rc : AMX_ERR_CUDA;
  }
  *out = p;
  return AMX_OK;
}

// The potential of `rho` (stored grid, mapped onto the solve grid) into p->fout.
template <typename T>
int potential(GravPlan* p, const T* rho, double G, const int* active, cudaStream_t s) {
  using C = typename Cplx<T>::type;
  const GravGrid& g = p->g;
  const long long nsolve = ipow_ll(g.M, g.dim);
  const long long nreal = ipow_ll(g.E, g.dim);
  const long long ncplx = ipow_ll(g.E, g.dim - 1) * (g.E / 2 + 1);
  const int grid = grid_for(nsolve, p->num_sms);
  if (p->periodic) {
    k_density_mean<T><<<kSumBlocks, kGThreads, 0, s>>>(rho, g, p->partial, p->counter, p->mean, active);
    k_density_pack<T><<<grid, kGThreads, 0, s>>>(rho, g, p->mean, static_cast<T*>(p->fin), active);
  } else {
    k_density_pack<T><<<grid, kGThreads, 0, s>>>(rho, g, nullptr, static_cast<T*>(p->fin), active);
  }
  int rc = cuda_ok(cudaGetLastError());
  rc |= fft_ok(cufftSetStream(p->fwd, s));
  rc |= fft_ok(cufftSetStream(p->inv, s));
  if (rc) return rc;
  if (sizeof(T) == 4) {
    rc = fft_ok(cufftExecR2C(p->fwd, static_cast<cufftReal*>(p->fin), static_cast<cufftComplex*>(p->spec)));
  } else {
    rc = fft_ok(cufftExecD2Z(p->fwd, static_cast<cufftDoubleReal*>(p->fin), static_cast<cufftDoubleComplex*>(p->spec)));
  }
  if (rc) return rc;
  const double inv_total = 1.0 / (double)nreal;
  const int cgrid = grid_for(ncplx, p->num_sms);
  if (p->periodic) {
    k_green_periodic<C><<<cgrid, kGThreads, 0, s>>>(static_cast<C*>(p->spec), g, p->dx, G, inv_total, active);
  } else {
    const double f = G * std::pow(p->dx, g.dim) * inv_total;
    k_green_open<C><<<cgrid, kGThreads, 0, s>>>(static_cast<C*>(p->spec), static_cast<const C*>(p->kspec), ncplx, f,
                                                active);
  }
  rc = cuda_ok(cudaGetLastError());
  if (rc) return rc;
  if (sizeof(T) == 4) {
    rc = fft_ok(cufftExecC2R(p->inv, static_cast<cufftComplex*>(p->spec), static_cast<cufftReal*>(p->fout)));
  } else {
    rc = fft_ok(cufftExecZ2D(p->inv, static_cast<cufftDoubleComplex*>(p->spec), static_cast<cufftDoubleReal*>(p->fout)));
  }
  return rc;
}

template <typename T, int DIM>
int launch_source(GravPlan* p, const T* old, T* state, const FVControl* ctl, double dt_scale, double gamma,
                  cudaStream_t s) {
  GravSrc<T> a{};
  a.old = old;
  a.state = state;
  a.phi = static_cast<const T*>(p->fout);
  a.g = p->g;
  a.nc = p->ncells;
  a.ctl = ctl;
  a.dt_scale = dt_scale;
  a.dx = p->dx;
  a.gamma = gamma;
  a.version = p->version;
  a.lm = p->lm;
  a.split = p->split;
  a.first_order = p->first_order;
  a.limiter = p->limiter;
  const int grid = grid_for(p->ncells, p->num_sms);
  if (p->rs == AMX_LAX_FRIEDRICHS) k_grav_source<T, DIM, RS_LF><<<grid, kGThreads, 0, s>>>(a);
  else if (p->rs == AMX_HLL) k_grav_source<T, DIM, RS_HLL><<<grid, kGThreads, 0, s>>>(a);
  else k_grav_source<T, DIM, RS_HLLC><<<grid, kGThreads, 0, s>>>(a);
  return cuda_ok(cudaGetLastError());
}

template <typename T>
int apply_t(GravPlan* p, const T* old, T* state, const FVControl* ctl, double dt_scale, const amx_params& prm,
            cudaStream_t s) {
  int rc = potential<T>(p, old, prm.gravitational_constant, &ctl->active, s);
  if (rc) return rc;
  switch (p->g.dim) {
    case 1: return launch_source<T, 1>(p, old, state, ctl, dt_scale, prm.gamma, s);
    case 2: return launch_source<T, 2>(p, old, state, ctl, dt_scale, prm.gamma, s);
    default: return launch_source<T, 3>(p, old, state, ctl, dt_scale, prm.gamma, s);
  }
}

bool all_periodic(const amx_config& c) {
  for (int k = 0; k < c.dimensionality; ++k)
    if (c.bc_lo[k] != AMX_BC_PERIODIC || c.bc_hi[k] != AMX_BC_PERIODIC) return false;
  return true;
}

}  // namespace

int grav_plan_create(const amx_config& c, GravPlan** out) {
  GravGrid g{};
  g.dim = c.dimensionality;
  g.n = c.num_cells;
  g.roll = c.boundary_handling == AMX_PERIODIC_ROLL;
  g.goff = g.roll ? 0 : 2;
  g.M = g.n + 2 * g.goff;
  const bool periodic = all_periodic(c);
  g.E = periodic ? g.M : 2 * g.M;
  for (int k = 0; k < 3; ++k) g.bc[k] = AxisBC{c.bc_lo[k], c.bc_hi[k]};
  const long long ncells = ipow_ll(c.num_cells, c.dimensionality);
  int rc = solver_create(g, c.grid_spacing, periodic, c.dtype, c.dimensionality + 2, ncells, out);
  if (rc) return rc;
  GravPlan* p = *out;
  p->version = c.self_gravity_version;
  p->rs = c.riemann_solver;
  p->lm = c.riemann_solver == AMX_HLLC_LM;
  p->split = c.split;
  p->first_order = c.first_order_fallback;
  p->limiter = c.limiter;
  return AMX_OK;
}

void grav_plan_destroy(GravPlan* p) {
  if (!p) return;
  if (p->have_fwd) cufftDestroy(p->fwd);
  if (p->have_inv) cufftDestroy(p->inv);
  if (p->mem) cudaFree(p->mem);
  delete p;
}

size_t grav_plan_bytes(const GravPlan* p) { return p ? p->bytes : 0; }
void* grav_old_state(GravPlan* p) { return p ? p->old : nullptr; }

int grav_apply(GravPlan* p, const void* old_state, void* state, const FVControl* ctl, double dt_scale,
               const amx_params& prm, cudaStream_t s) {
  if (!p || !old_state || !state || !ctl) return AMX_ERR_INVALID_ARG;
  if (p->dtype == AMX_F32)
    return apply_t<float>(p, static_cast<const float*>(old_state), static_cast<float*>(state), ctl, dt_scale, prm, s);
  return apply_t<double>(p, static_cast<const double*>(old_state), static_cast<double*>(state), ctl, dt_scale, prm, s);
}

int grav_advance(FVControl* ctl, double* dt_hist, int* it_hist, long long max_hist, int mhd, cudaStream_t s) {
  k_grav_advance<<<1, 32, 0, s>>>(ctl, dt_hist, it_hist, max_hist, mhd);
  return cuda_ok(cudaGetLastError());
}

}  // namespace amx

// ====================================================================== ABI

struct amx_poisson {
  amx::GravPlan* plan;
};

extern "C" {

int amx_poisson_create(int32_t dimensionality, int32_t num_cells, double grid_spacing, int32_t periodic,
                       int32_t dtype, amx_poisson** out) {
  if (!out) return AMX_ERR_INVALID_ARG;
  *out = nullptr;
  if (dimensionality < 1 || dimensionality > 3 || num_cells < 2 || !(grid_spacing > 0.0)) return AMX_ERR_INVALID_ARG;
  if (dtype != AMX_F32 && dtype != AMX_F64) return AMX_ERR_INVALID_ARG;
  amx::GravGrid g{};
  g.dim = dimensionality;
  g.n = num_cells;
  g.goff = 0;
  g.M = num_cells;
  g.E = periodic ? num_cells : 2 * num_cells;
  g.roll = 0;
  for (int k = 0; k < 3; ++k) g.bc[k] = amx::AxisBC{AMX_BC_PERIODIC, AMX_BC_PERIODIC};
  amx::GravPlan* p = nullptr;
  int rc = amx::solver_create(g, grid_spacing, periodic != 0, dtype, 0, amx::ipow_ll(num_cells, dimensionality), &p);
  if (rc) return rc;
  amx_poisson* h = new (std::nothrow) amx_poisson{p};
  if (!h) { amx::grav_plan_destroy(p); return AMX_ERR_INVALID_ARG; }
  *out = h;
  return AMX_OK;
}

int amx_poisson_destroy(amx_poisson* h) {
  if (!h) return AMX_OK;
  amx::grav_plan_destroy(h->plan);
  delete h;
  return AMX_OK;
}

int amx_poisson_solve(amx_poisson* h, const void* density, void* potential, double G, void* stream) {
  if (!h || !density || !potential) return AMX_ERR_INVALID_ARG;
  amx::GravPlan* p = h->plan;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long total = amx::ipow_ll(p->g.M, p->g.dim);
  const int grid = amx::grid_for(total, p->num_sms);
  int rc;
  if (p->dtype == AMX_F32) {
    rc = amx::potential<float>(p, static_cast<const float*>(density), G, nullptr, s);
    if (!rc) amx::k_crop<float><<<grid, amx::kGThreads, 0, s>>>(static_cast<const float*>(p->fout), p->g,
                                                                  static_cast<float*>(potential));
  } else {
    rc = amx::potential<double>(p, static_cast<const double*>(density), G, nullptr, s);
    if (!rc) amx::k_crop<double><<<grid, amx::kGThreads, 0, s>>>(static_cast<const double*>(p->fout), p->g,
                                                                   static_cast<double*>(potential));
  }
  if (rc) return rc;
  return amx::cuda_ok(cudaGetLastError());
}

}  // extern "C"
