// Measurement utility: the FP32 FMA throughput of this GPU, the compute roof
// of the FD WENO kernel (no reference counterpart).
#include <cuda_runtime.h>

#include "../../include/amx.h"

namespace {

constexpr int kChains = 8;

// kChains independent FMA chains per thread, `iters` rounds; the result is
// stored only under a condition the data never meets, so nothing is elided.
__global__ void __launch_bounds__(256) fma_probe_kernel(float* out, int iters, float a, float b) {
  float x[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) x[i] = (float)(threadIdx.x + i) * 1e-7f;
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = fmaf(x[i], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += x[i];
  if (s == 123456.0f) out[blockIdx.x] = s;
}

}  // namespace

extern "C" int amx_probe_fp32_fma(double* tflops, void* stream) {
  if (!tflops) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return AMX_ERR_CUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  float* out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * 65536) != cudaSuccess) return AMX_ERR_CUDA;
  const int blocks = sms * 8, iters = 1 << 14;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // a contraction near 1 keeps the chains finite
  fma_probe_kernel<<<blocks, 256, 0, s>>>(out, 256, 0.999999f, 1e-7f);
  cudaEventRecord(e0, s);
  fma_probe_kernel<<<blocks, 256, 0, s>>>(out, iters, 0.999999f, 1e-7f);
  cudaEventRecord(e1, s);
  int rc = cudaEventSynchronize(e1) == cudaSuccess ? AMX_OK : AMX_ERR_CUDA;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  *tflops = 2.0 * kChains * (double)iters * blocks * 256 / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return rc;
}
