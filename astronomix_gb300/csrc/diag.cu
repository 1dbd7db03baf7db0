// FP64 conservation sums and max |div B| (astronomix/_fluid_equations/
// total_quantities.py:31-176, time_integration.py:507-522).
#include <cuda_runtime.h>

#include "../../include/amx.h"
#include "amx_common.cuh"
#include "fv_physics.cuh"

namespace amx {

// out[0] sum rho, out[1] sum E_gas, out[2] sum 0.5 rho u^2, out[3] sum p/(g-1),
// out[4] (as bits) max |div B|
template <typename T, int DIM>
__global__ void diag_kernel(const T* __restrict__ s, int n, long long nc, int b_row, int face_b, double dx,
                            double gamma, double* out) {
  __shared__ double red[32];
  double m = 0.0, e = 0.0, k = 0.0, in = 0.0, dv = 0.0;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += (long long)gridDim.x * blockDim.x) {
    const T rho = s[c];
    const T p = s[(DIM + 1) * nc + c];
    T q[DIM + 2];
    q[0] = rho;
    for (int a = 1; a <= DIM; ++a) q[a] = s[a * nc + c];
    q[DIM + 1] = p;
    // FD states always carry 3 velocity rows; the 3D absolute velocity adds 1e-20
    const T u = abs_velocity<T, DIM>(q);
    const T g = T(gamma);
    m += (double)rho;
    e += (double)total_energy(rho, u, p, g);
    k += (double)(T(0.5) * rho * (u * u));
    in += (double)(p / (g - T(1)));
    if (b_row >= 0) {
      int ic[3] = {0, 0, 0};
      if (DIM == 2) { ic[0] = (int)(c / n); ic[1] = (int)(c % n); }
      if (DIM == 3) { ic[2] = (int)(c % n); ic[1] = (int)((c / n) % n); ic[0] = (int)(c / ((long long)n * n)); }
      double div = 0.0;
      for (int a = 0; a < DIM; ++a) {
        const T* f = s + (long long)(b_row + a) * nc;
        int jp[3] = {ic[0], ic[1], ic[2]}, jm[3] = {ic[0], ic[1], ic[2]};
        if (face_b) {
          // 6th-order interface difference (_differencing.py:9-51)
          double acc = 0.0;
          const double c1 = 75.0 / 64.0, c2 = -25.0 / 384.0, c3 = 3.0 / 640.0;
          auto at = [&](int off) {
            int j[3] = {ic[0], ic[1], ic[2]};
            j[a] = wrap(j[a] + off, n);
            return (double)f[((long long)j[0] * n + j[1]) * n + j[2]];
          };
          acc = c1 * (at(0) - at(-1)) + c2 * (at(1) - at(-2)) + c3 * (at(2) - at(-3));
          div += acc / dx;
        } else {
          jp[a] = wrap(jp[a] + 1, n);
          jm[a] = wrap(jm[a] - 1, n);
          long long cp = (DIM == 2) ? (long long)jp[0] * n + jp[1] : ((long long)jp[0] * n + jp[1]) * n + jp[2];
          long long cm = (DIM == 2) ? (long long)jm[0] * n + jm[1] : ((long long)jm[0] * n + jm[1]) * n + jm[2];
          div += ((double)f[cp] - (double)f[cm]) / (2.0 * dx);
        }
      }
      dv = fmax(dv, fabs(div));
    }
  }
  // block sums
  auto bsum = [&](double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
      r = (threadIdx.x < (blockDim.x + 31) / 32) ? red[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    return r;
  };
  const double sm = bsum(m), se = bsum(e), sk = bsum(k), si = bsum(in);
  const double md = block_max<double>(dv, red);
  if (threadIdx.x == 0) {
    atomicAdd(&out[0], sm);
    atomicAdd(&out[1], se);
    atomicAdd(&out[2], sk);
    atomicAdd(&out[3], si);
    atomic_max_nonneg(reinterpret_cast<unsigned long long*>(&out[4]), md);
  }
}

template <typename T>
static int launch_diag(int dim, const void* state, int n, long long nc, int b_row, int face_b, double dx,
                       double gamma, double* out, cudaStream_t s) {
  const int threads = 256;
  const int blocks = (int)((nc + threads - 1) / threads < 4096 ? (nc + threads - 1) / threads : 4096);
  const T* st = static_cast<const T*>(state);
  if (dim == 1) diag_kernel<T, 1><<<blocks, threads, 0, s>>>(st, n, nc, -1, 0, dx, gamma, out);
  else if (dim == 2) diag_kernel<T, 2><<<blocks, threads, 0, s>>>(st, n, nc, b_row, face_b, dx, gamma, out);
  else diag_kernel<T, 3><<<blocks, threads, 0, s>>>(st, n, nc, b_row, face_b, dx, gamma, out);
  return cudaGetLastError() == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
}

}  // namespace amx

extern "C" int amx_diag_sums_raw(const amx_config* cfg, const void* state, double gamma, double* out_dev,
                                 void* stream) {
  if (!cfg || !state || !out_dev) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int d = cfg->dimensionality, n = cfg->num_cells;
  long long nc = 1;
  for (int i = 0; i < d; ++i) nc *= n;
  int b_row = -1, face_b = 0;
  if (cfg->mhd) {
    if (cfg->solver_mode == AMX_FINITE_DIFFERENCE) { b_row = 8; face_b = 1; }
    else b_row = d + 2;
  }
  if (cudaMemsetAsync(out_dev, 0, 5 * sizeof(double), s) != cudaSuccess) return AMX_ERR_CUDA;
  // FD states carry three velocity rows: treat them as 3D (they are)
  if (cfg->dtype == AMX_F32)
    return amx::launch_diag<float>(d, state, n, nc, b_row, face_b, cfg->grid_spacing, gamma, out_dev, s);
  return amx::launch_diag<double>(d, state, n, nc, b_row, face_b, cfg->grid_spacing, gamma, out_dev, s);
}
