// Host-side lookup of the batched FV kernel instantiations.
#pragma once
#include <stddef.h>

namespace amx {

struct BatchKernelInfo {
  const void* fn;  // __global__ function
  size_t smem;     // dynamic shared memory per block
  int variant;     // tile shape (TileV)
  int tile0, tile1;
};

// riemann family 0 = HLL, 1 = HLLC (and HLLC-LM); 2D only.  Returns false
// for combinations that are not instantiated.
bool fv_batch_kernel_f32(int dim, int rs, bool mhd, int variant, BatchKernelInfo* out);
bool fv_batch_kernel_f64(int dim, int rs, bool mhd, int variant, BatchKernelInfo* out);
// variants 1 and 2 of the float kernels (own translation unit)
bool fv_batch_kernel_f32_alt(int dim, int rs, bool mhd, int variant, BatchKernelInfo* out);

}  // namespace amx
