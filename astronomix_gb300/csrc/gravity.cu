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
#include "gravity_source.cuh"

namespace amx {
// instantiated in gravity_f32.cu (approximate FP32 division and square root)
extern template int grav_source_launch<float>(const GravSrc<float>&, int, int, cudaStream_t);
}  // namespace amx

namespace amx {

namespace {

constexpr int kSumBlocks = 304;

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

__device__ __forceinline__ long long ext_index(const GravGrid& g, const int* p) { return grav_ext_index(g, p); }

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

// Periodic Green's function (_poisson_solver.py:86-113) on the half spectrum
// for G = 1, times `scale` (the inverse transform's 1 / E^d), computed once
// per solver: the wave numbers are 2 pi fftfreq(E, dx), -4 pi / k^2 and
// -1 / (4 pi) at k = 0.
template <typename R>
__global__ void __launch_bounds__(kGThreads) k_green_periodic_init(R* green, GravGrid g, double dx, double scale) {
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
    const double gr = (k2 > 1e-12) ? (-4.0 * pi) / k2 : -1.0 / (4.0 * pi);
    green[e] = R(gr * scale);
  }
}

// The spectrum times the real Green's function times G (periodic).
template <typename C, typename R>
__global__ void __launch_bounds__(kGThreads) k_spec_scale(C* spec, const R* __restrict__ green, long long total, R G,
                                                          const int* active) {
  if (active && !*(volatile const int*)active) return;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const R f = green[e] * G;
    C z = spec[e];
    z.x = z.x * f;
    z.y = z.y * f;
    spec[e] = z;
  }
}

// The spectrum times the isolated kernel's spectrum (G = 1, scaled by
// dx^d / E^d once per solver) times G (open boundaries).
template <typename C, typename R>
__global__ void __launch_bounds__(kGThreads) k_spec_mul(C* spec, const C* __restrict__ kspec, long long total, R G,
                                                        const int* active) {
  if (active && !*(volatile const int*)active) return;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const C a = spec[e], b = kspec[e];
    C z;
    z.x = (a.x * b.x - a.y * b.y) * G;
    z.y = (a.x * b.y + a.y * b.x) * G;
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
__global__ void k_convert_spectrum(const D* in, C* out, long long total, double scale) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    C z;
    z.x = in[e].x * scale;
    z.y = in[e].y * scale;
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


inline int cuda_ok(cudaError_t e) { return e == cudaSuccess ? AMX_OK : AMX_ERR_CUDA; }
inline int fft_ok(cufftResult r) { return r == CUFFT_SUCCESS ? AMX_OK : AMX_ERR_CUDA; }
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
inline int grid_for(long long work, int num_sms) { return grav_grid_for(work, num_sms); }

}  // namespace

struct GravPlan {
  GravGrid g{};
  int dtype = AMX_F32;
  bool periodic = true;
  double dx = 1.0;
  int version = AMX_DONOR_ACCOUNTING;
  int rs = AMX_HLL;
  int lm = 0, am = 0, split = 0, first_order = 0, limiter = AMX_MINMOD;
  long long ncells = 0;
  int num_sms = 1;
  cufftHandle fwd = 0, inv = 0;
  bool have_fwd = false, have_inv = false;
  // open boundaries in 2D / 3D: the transforms skip the zero half of the
  // padded grid along x (the density lives in planes x < M, the potential is
  // read there): a (d-1)-dimensional R2C / C2R over the planes x < M and a
  // strided 1D C2C along x over the whole half spectrum
  bool pruned = false;
  cufftHandle outer = 0;
  bool have_outer = false;
  void* spec2 = nullptr;  // pruned: the x-transformed half spectrum (spec keeps its planes x >= M zero)
  unsigned char* mem = nullptr;
  size_t bytes = 0;
  void* fin = nullptr;    // FFT input (E^d real; pruned: the planes x < M, M E^(d-1))
  void* fout = nullptr;   // inverse transform, same shape: the potential in its solve-grid corner
  void* spec = nullptr;   // half spectrum
  void* kspec = nullptr;  // the Green's function's half spectrum for G = 1, with the inverse
                          // transform's scale: real (periodic) or complex (open)
  void* old = nullptr;    // run: gas rows of the state before a gas update
  void* eacc = nullptr;   // run: [ncells] energy source summed over the axes
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
  p->pruned = !periodic && g.dim >= 2;
  // pruned: the real arrays hold the planes x < M only
  const long long nreal_buf = p->pruned ? (long long)g.M * ipow_ll(g.E, g.dim - 1) : nreal;
  size_t off = 0;
  const size_t o_in = off; off = align256(off + elem * nreal_buf);
  const size_t o_out = off; off = align256(off + elem * nreal_buf);
  const size_t o_sp = off; off = align256(off + 2 * elem * ncplx);
  const size_t o_sp2 = off; off = align256(off + (p->pruned ? 2 * elem * ncplx : 0));
  const size_t o_ks = off; off = align256(off + (periodic ? 1 : 2) * elem * ncplx);
  const size_t o_old = off; off = align256(off + elem * (size_t)old_rows * ncells);
  const size_t o_eacc = off; off = align256(off + (old_rows ? elem * (size_t)ncells : 0));
  const size_t o_part = off; off = align256(off + sizeof(double) * kSumBlocks);
  const size_t o_cnt = off; off = align256(off + sizeof(unsigned int));
  const size_t o_mean = off; off = align256(off + sizeof(double));
  p->bytes = off;
  if (cudaMalloc(&p->mem, off) != cudaSuccess) { delete p; return AMX_ERR_CUDA; }
  cudaMemset(p->mem, 0, off);
  p->fin = p->mem + o_in;
  p->fout = p->mem + o_out;
  p->spec = p->mem + o_sp;
  p->spec2 = p->pruned ? p->mem + o_sp2 : nullptr;
  p->kspec = p->mem + o_ks;
  p->old = old_rows ? p->mem + o_old : nullptr;
  p->eacc = old_rows ? p->mem + o_eacc : nullptr;
  p->partial = reinterpret_cast<double*>(p->mem + o_part);
  p->counter = reinterpret_cast<unsigned int*>(p->mem + o_cnt);
  p->mean = reinterpret_cast<double*>(p->mem + o_mean);
  int nn[3] = {g.E, g.E, g.E};
  int rc;
  if (!p->pruned) {
    rc = fft_ok(cufftPlanMany(&p->fwd, g.dim, nn, nullptr, 1, 0, nullptr, 1, 0,
                              dtype == AMX_F32 ? CUFFT_R2C : CUFFT_D2Z, 1));
    p->have_fwd = rc == AMX_OK;
    if (!rc) {
      rc = fft_ok(cufftPlanMany(&p->inv, g.dim, nn, nullptr, 1, 0, nullptr, 1, 0,
                                dtype == AMX_F32 ? CUFFT_C2R : CUFFT_Z2D, 1));
      p->have_inv = rc == AMX_OK;
    }
  } else {
    // (d-1)-dimensional transforms of the M planes x < M (contiguous planes)
    rc = fft_ok(cufftPlanMany(&p->fwd, g.dim - 1, nn, nullptr, 1, 0, nullptr, 1, 0,
                              dtype == AMX_F32 ? CUFFT_R2C : CUFFT_D2Z, g.M));
    p->have_fwd = rc == AMX_OK;
    if (!rc) {
      rc = fft_ok(cufftPlanMany(&p->inv, g.dim - 1, nn, nullptr, 1, 0, nullptr, 1, 0,
                                dtype == AMX_F32 ? CUFFT_C2R : CUFFT_Z2D, g.M));
      p->have_inv = rc == AMX_OK;
    }
    if (!rc) {
      // 1D along x, one transform per (y, kz) of the half spectrum
      const int S = (int)(ncplx / g.E);
      int ne[1] = {g.E};
      rc = fft_ok(cufftPlanMany(&p->outer, 1, ne, ne, S, 1, ne, S, 1, dtype == AMX_F32 ? CUFFT_C2C : CUFFT_Z2Z, S));
      p->have_outer = rc == AMX_OK;
    }
  }
  const double inv_total = 1.0 / (double)nreal;
  if (!rc && periodic) {
    if (dtype == AMX_F32)
      k_green_periodic_init<float><<<grid_for(ncplx, p->num_sms), kGThreads>>>(static_cast<float*>(p->kspec), g, dx,
                                                                               inv_total);
    else
      k_green_periodic_init<double><<<grid_for(ncplx, p->num_sms), kGThreads>>>(static_cast<double*>(p->kspec), g,
                                                                                dx, inv_total);
    rc = cuda_ok(cudaGetLastError());
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
        // the reference scales the cropped potential by dx^d (_poisson_solver.py:151)
        const double scale = std::pow(dx, g.dim) * inv_total;
        if (dtype == AMX_F32)
          k_convert_spectrum<cufftComplex, cufftDoubleComplex>
              <<<grid_for(ncplx, p->num_sms), kGThreads>>>(kc, static_cast<cufftComplex*>(p->kspec), ncplx, scale);
        else
          k_convert_spectrum<cufftDoubleComplex, cufftDoubleComplex>
              <<<grid_for(ncplx, p->num_sms), kGThreads>>>(kc, static_cast<cufftDoubleComplex*>(p->kspec), ncplx,
                                                           scale);
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
  if (p->pruned) rc |= fft_ok(cufftSetStream(p->outer, s));
  if (rc) return rc;
  if (sizeof(T) == 4) {
    rc = fft_ok(cufftExecR2C(p->fwd, static_cast<cufftReal*>(p->fin), static_cast<cufftComplex*>(p->spec)));
  } else {
    rc = fft_ok(cufftExecD2Z(p->fwd, static_cast<cufftDoubleReal*>(p->fin), static_cast<cufftDoubleComplex*>(p->spec)));
  }
  if (rc) return rc;
  // pruned: along x out of place, so that spec keeps its zero planes x >= M
  C* sp = static_cast<C*>(p->pruned ? p->spec2 : p->spec);
  if (p->pruned) {
    if (sizeof(T) == 4)
      rc = fft_ok(cufftExecC2C(p->outer, static_cast<cufftComplex*>(p->spec), reinterpret_cast<cufftComplex*>(sp),
                               CUFFT_FORWARD));
    else
      rc = fft_ok(cufftExecZ2Z(p->outer, static_cast<cufftDoubleComplex*>(p->spec),
                               reinterpret_cast<cufftDoubleComplex*>(sp), CUFFT_FORWARD));
    if (rc) return rc;
  }
  const int cgrid = grid_for(ncplx, p->num_sms);
  if (p->periodic)
    k_spec_scale<C, T><<<cgrid, kGThreads, 0, s>>>(sp, static_cast<const T*>(p->kspec), ncplx, T(G), active);
  else
    k_spec_mul<C, T><<<cgrid, kGThreads, 0, s>>>(sp, static_cast<const C*>(p->kspec), ncplx, T(G), active);
  rc = cuda_ok(cudaGetLastError());
  if (rc) return rc;
  if (p->pruned) {
    if (sizeof(T) == 4)
      rc = fft_ok(cufftExecC2C(p->outer, reinterpret_cast<cufftComplex*>(sp), reinterpret_cast<cufftComplex*>(sp),
                               CUFFT_INVERSE));
    else
      rc = fft_ok(cufftExecZ2Z(p->outer, reinterpret_cast<cufftDoubleComplex*>(sp),
                               reinterpret_cast<cufftDoubleComplex*>(sp), CUFFT_INVERSE));
    if (rc) return rc;
  }
  if (sizeof(T) == 4) {
    rc = fft_ok(cufftExecC2R(p->inv, reinterpret_cast<cufftComplex*>(sp), static_cast<cufftReal*>(p->fout)));
  } else {
    rc = fft_ok(cufftExecZ2D(p->inv, reinterpret_cast<cufftDoubleComplex*>(sp), static_cast<cufftDoubleReal*>(p->fout)));
  }
  return rc;
}

template <typename T>
int apply_t(GravPlan* p, const T* old, T* state, const FVControl* ctl, double dt_scale, const amx_params& prm,
            cudaStream_t s) {
  int rc = potential<T>(p, old, prm.gravitational_constant, &ctl->active, s);
  if (rc) return rc;
  GravSrc<T> a{};
  a.old = old;
  a.state = state;
  a.phi = static_cast<const T*>(p->fout);
  a.eacc = static_cast<T*>(p->eacc);
  a.g = p->g;
  a.nc = p->ncells;
  a.ctl = ctl;
  a.dt_scale = dt_scale;
  a.dx = p->dx;
  a.gamma = prm.gamma;
  a.version = p->version;
  a.lm = p->lm;
  a.am = p->am;
  a.split = p->split;
  a.first_order = p->first_order;
  a.limiter = p->limiter;
  return grav_source_launch<T>(a, p->rs, p->num_sms, s);
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
  p->am = (c.riemann_solver == AMX_AM_HLLC) ? 1 : (c.riemann_solver == AMX_HYBRID_HLLC ? 2 : 0);
  p->split = c.split;
  p->first_order = c.first_order_fallback;
  p->limiter = c.limiter;
  return AMX_OK;
}

void grav_plan_destroy(GravPlan* p) {
  if (!p) return;
  if (p->have_fwd) cufftDestroy(p->fwd);
  if (p->have_inv) cufftDestroy(p->inv);
  if (p->have_outer) cufftDestroy(p->outer);
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
