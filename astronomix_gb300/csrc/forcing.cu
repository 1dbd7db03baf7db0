// Turbulent forcing (_physics_modules/_turbulent_forcing/_turbulent_forcing.py:15-128):
// a solenoidal random velocity field with the spectrum k^6 exp(-8 k / k_p),
// k_p = 4 pi / L, drawn in Fourier space, transformed back with cuFFT, and
// added to the velocities with the amplitude that injects
// energy_injection_rate * dt of kinetic energy.
//
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), keyed by
// the seed, counter (mode, component, step low, step high); two uniforms per
// complex draw, a normal pair by Box-Muller.  The reference draws from
// jax.random (threefry), which has no counterpart here: the spectrum,
// projection, normalisation and amplitude are the reference's, the random
// stream is this generator's.
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include <cmath>
#include <new>

#include "../../include/amx.h"
#include "amx_common.cuh"
#include "forcing.h"

namespace amx {

namespace {

constexpr int kFThreads = 256;
constexpr int kFSumBlocks = 304;

struct Philox4 {
  uint32_t x[4];
};

// Philox4x32-10: ten rounds of two 32x32->64 multiplies, the key bumped by
// the Weyl constants between rounds (the published algorithm).
__device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                                 uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += W0;
      k1 += W1;
    }
    const uint64_t p0 = (uint64_t)M0 * c0;
    const uint64_t p1 = (uint64_t)M1 * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
  }
  Philox4 r;
  r.x[0] = c0;
  r.x[1] = c1;
  r.x[2] = c2;
  r.x[3] = c3;
  return r;
}

__device__ __forceinline__ double block_sum_f(double v, double* scratch) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) r += scratch[w];
  return r;  // valid in thread 0
}

template <typename T> struct FCplx;
template <> struct FCplx<float> { using type = cufftComplex; };
template <> struct FCplx<double> { using type = cufftDoubleComplex; };

// The three solenoidal Fourier fields of one step (_turbulent_forcing.py:15-63),
// computed in R (FP64 for FP64 states, FP32 for FP32 ones: GB300's FP64
// transcendentals would dominate the forcing otherwise); the inverse
// transform's 1 / n^3 is applied by the readers.
template <typename C, typename R>
__global__ void __launch_bounds__(kFThreads) k_force_spectrum(C* W, int n, double box, unsigned long long seed,
                                                              const long long* steps, const int* active) {
  if (!*(volatile const int*)active) return;
  const long long n3 = (long long)n * n * n;
  const unsigned long long step = (unsigned long long)*(volatile const long long*)steps;
  const R pi = R(3.141592653589793);
  const R val = R(1.0 / ((double)n * (box / n)));
  const R kpk = R(4.0 * 3.141592653589793 / box);
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n3; m += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(m / ((long long)n * n)), j = (int)((m / n) % n), l = (int)(m % n);
    auto freq = [&](int q) { return R((q <= (n - 1) / 2) ? q : q - n) * val; };
    const R kx = R(2) * pi * freq(i), ky = R(2) * pi * freq(j), kz = R(2) * pi * freq(l);
    const R k2 = kx * kx + ky * ky + kz * kz;
    const R kk = sqrt(k2);
    const R Pk = pow(kk, R(6)) * exp(R(-8) * kk / kpk);
    const R sq = sqrt(Pk);
    R re[3], im[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const Philox4 r = philox4x32_10((uint32_t)m, (uint32_t)c, (uint32_t)step, (uint32_t)(step >> 32), k0, k1);
      const R u1 = R(((double)r.x[0] + 1.0) * 2.3283064365386963e-10);  // 2^-32
      const R u2 = R((double)r.x[1] * 2.3283064365386963e-10);
      const R rr = sqrt(R(-2) * log(u1));
      const R th = R(2) * pi * u2;
      re[c] = m == 0 ? R(0) : sq * (rr * cos(th));
      im[c] = m == 0 ? R(0) : sq * (rr * sin(th));
    }
    // project out the compressive part: w -= k (k . w) / k^2
    const R k2s = (k2 == R(0)) ? R(1) : k2;
    R dre = (kx * re[0] + ky * re[1] + kz * re[2]) / k2s;
    R dim = (kx * im[0] + ky * im[1] + kz * im[2]) / k2s;
    if (m == 0) dre = dim = R(0);
    const R kv[3] = {kx, ky, kz};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      C z;
      z.x = re[c] - kv[c] * dre;
      z.y = im[c] - kv[c] * dim;
      W[c * n3 + m] = z;
    }
  }
}

// The amplitude (_turbulent_forcing.py:82-110): a = 1/2 sum rho |w|^2,
// b = sum rho v.w, c = -Edot dt / dV, amp = (-b + sqrt(b^2 - 4ac)) / 2a (0
// when the discriminant is negative or a vanishes).  FP64 sums, per-block
// partials added in block order by the last block (deterministic).
template <typename T, typename C>
__global__ void __launch_bounds__(kFThreads) k_force_amplitude(const T* P, const C* W, long long n3, double* partial,
                                                               unsigned int* counter, double* amp, const double* dt,
                                                               double edot, double dV, const int* active) {
  __shared__ double scratch[32];
  __shared__ bool last;
  if (!*(volatile const int*)active) return;
  const double inv = 1.0 / (double)n3;
  double sa = 0.0, sb = 0.0;
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n3; m += (long long)gridDim.x * blockDim.x) {
    const double rho = P[m];
    const double wx = (double)W[m].x * inv, wy = (double)W[n3 + m].x * inv, wz = (double)W[2 * n3 + m].x * inv;
    sa += rho * (wx * wx + wy * wy + wz * wz);
    sb += rho * (double)P[n3 + m] * wx + rho * (double)P[2 * n3 + m] * wy + rho * (double)P[3 * n3 + m] * wz;
  }
  sa = block_sum_f(sa, scratch);
  sb = block_sum_f(sb, scratch);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = sa;
    partial[gridDim.x + blockIdx.x] = sb;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double a = 0.0, b = 0.0;
    for (unsigned int k = 0; k < gridDim.x; ++k) {
      a += ((volatile double*)partial)[k];
      b += ((volatile double*)partial)[gridDim.x + k];
    }
    a = 0.5 * a;
    const double c = -edot * *(volatile const double*)dt / dV;
    const double disc = b * b - 4.0 * a * c;
    *amp = (disc >= 0.0 && fabs(a) > 1e-10) ? (-b + sqrt(disc)) / (2.0 * a) : 0.0;
    *counter = 0u;
  }
}

template <typename T, typename C>
__global__ void __launch_bounds__(kFThreads) k_force_apply(T* P, const C* W, long long n3, const double* amp,
                                                           const int* active) {
  if (!*(volatile const int*)active) return;
  const T a = T(*(volatile const double*)amp);
  const T inv = T(1.0 / (double)n3);
  for (long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x; m < n3; m += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) P[(1 + c) * n3 + m] = P[(1 + c) * n3 + m] + a * (T(W[c * n3 + m].x) * inv);
  }
}

inline int cuda_ok(cudaError_t e) { return e == cudaSuccess ? AMX_OK : AMX_ERR_CUDA; }
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

struct ForcingPlan {
  int n = 0;
  int dtype = AMX_F32;
  double box = 1.0;
  double dx = 1.0;
  long long n3 = 0;
  int num_sms = 1;
  cufftHandle plan = 0;
  bool have_plan = false;
  unsigned char* mem = nullptr;
  size_t bytes = 0;
  void* W = nullptr;  // [3][n^3] complex
  double* partial = nullptr;
  unsigned int* counter = nullptr;
  double* amp = nullptr;
};

int forcing_plan_create(const amx_config& c, ForcingPlan** out) {
  if (c.dimensionality != 3) return AMX_ERR_UNSUPPORTED;
  ForcingPlan* f = new (std::nothrow) ForcingPlan();
  if (!f) return AMX_ERR_INVALID_ARG;
  f->n = c.num_cells;
  f->dtype = c.dtype;
  f->box = c.box_size;
  f->dx = c.grid_spacing;
  f->n3 = (long long)c.num_cells * c.num_cells * c.num_cells;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&f->num_sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t celem = c.dtype == AMX_F32 ? sizeof(cufftComplex) : sizeof(cufftDoubleComplex);
  size_t off = 0;
  const size_t o_w = off; off = align256(off + 3 * celem * (size_t)f->n3);
  const size_t o_p = off; off = align256(off + sizeof(double) * 2 * kFSumBlocks);
  const size_t o_c = off; off = align256(off + sizeof(unsigned int));
  const size_t o_a = off; off = align256(off + sizeof(double));
  f->bytes = off;
  if (cudaMalloc(&f->mem, off) != cudaSuccess) { delete f; return AMX_ERR_CUDA; }
  cudaMemset(f->mem, 0, off);
  f->W = f->mem + o_w;
  f->partial = reinterpret_cast<double*>(f->mem + o_p);
  f->counter = reinterpret_cast<unsigned int*>(f->mem + o_c);
  f->amp = reinterpret_cast<double*>(f->mem + o_a);
  int nn[3] = {f->n, f->n, f->n};
  const int n3 = (int)f->n3;
  if (cufftPlanMany(&f->plan, 3, nn, nullptr, 1, n3, nullptr, 1, n3, c.dtype == AMX_F32 ? CUFFT_C2C : CUFFT_Z2Z,
                    3) != CUFFT_SUCCESS) {
    forcing_plan_destroy(f);
    return AMX_ERR_CUDA;
  }
  f->have_plan = true;
  if (cudaDeviceSynchronize() != cudaSuccess) { forcing_plan_destroy(f); return AMX_ERR_CUDA; }
  *out = f;
  return AMX_OK;
}

void forcing_plan_destroy(ForcingPlan* f) {
  if (!f) return;
  if (f->have_plan) cufftDestroy(f->plan);
  if (f->mem) cudaFree(f->mem);
  delete f;
}

size_t forcing_plan_bytes(const ForcingPlan* f) { return f ? f->bytes : 0; }

namespace {

template <typename T>
int apply_t(ForcingPlan* f, T* P, const double* dt, const int* active, const long long* steps, const amx_params& prm,
            cudaStream_t s) {
  using C = typename FCplx<T>::type;
  C* W = static_cast<C*>(f->W);
  const long long b = (f->n3 + kFThreads - 1) / kFThreads;
  const int grid = (int)(b < (long long)f->num_sms * 8 ? b : (long long)f->num_sms * 8);
  k_force_spectrum<C, T><<<grid, kFThreads, 0, s>>>(W, f->n, f->box, (unsigned long long)prm.forcing_seed, steps,
                                                     active);
  if (cudaGetLastError() != cudaSuccess) return AMX_ERR_CUDA;
  if (cufftSetStream(f->plan, s) != CUFFT_SUCCESS) return AMX_ERR_CUDA;
  cufftResult r;
  if (sizeof(T) == 4)
    r = cufftExecC2C(f->plan, reinterpret_cast<cufftComplex*>(W), reinterpret_cast<cufftComplex*>(W), CUFFT_INVERSE);
  else
    r = cufftExecZ2Z(f->plan, reinterpret_cast<cufftDoubleComplex*>(W), reinterpret_cast<cufftDoubleComplex*>(W),
                     CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) return AMX_ERR_CUDA;
  const double dV = f->dx * f->dx * f->dx;
  k_force_amplitude<T, C><<<kFSumBlocks, kFThreads, 0, s>>>(P, W, f->n3, f->partial, f->counter, f->amp, dt,
                                                            prm.energy_injection_rate, dV, active);
  k_force_apply<T, C><<<grid, kFThreads, 0, s>>>(P, W, f->n3, f->amp, active);
  return cuda_ok(cudaGetLastError());
}

}  // namespace

int forcing_apply(ForcingPlan* f, void* state, const double* dt, const int* active, const long long* steps,
                  const amx_params& prm, cudaStream_t s) {
  if (!f || !state || !dt || !active || !steps) return AMX_ERR_INVALID_ARG;
  if (f->dtype == AMX_F32) return apply_t<float>(f, static_cast<float*>(state), dt, active, steps, prm, s);
  return apply_t<double>(f, static_cast<double*>(state), dt, active, steps, prm, s);
}

}  // namespace amx
