// Host-side lookup of the FV kernel instantiations (one TU per precision).
#pragma once
#include <stddef.h>

namespace amx {

struct FVKernelInfo {
  const void* fn;      // __global__ function
  size_t smem;         // dynamic shared memory per block
};

// riemann family: 0 = HLL, 1 = HLLC (and HLLC-LM), 3 = Lax-Friedrichs
bool fv_kernel_f32(int dim, int rs, bool mhd, FVKernelInfo* out);
bool fv_kernel_f64(int dim, int rs, bool mhd, FVKernelInfo* out);

}  // namespace amx
