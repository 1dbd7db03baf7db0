// Host-side lookup of the FV kernel instantiations (one TU per precision).
#pragma once
#include <stddef.h>

namespace amx {

struct FVKernelInfo {
  const void* fn;      // __global__ function
  size_t smem;         // dynamic shared memory per block
  size_t smem_pp;      // extra shared memory with the VAN_ALBADA_PP limiter
};

// riemann family: 0 = HLL, 1 = HLLC (and HLLC-LM), 3 = Lax-Friedrichs,
// 4 = HLLC with the AM_HLLC / HYBRID_HLLC compression switch (fv_riemann_family)
// scheme: FV_UNSPLIT, FV_SPLIT or FV_UNSPLIT_PP (fv_kernels.cuh)
bool fv_kernel_f32(int dim, int rs, bool mhd, int scheme, FVKernelInfo* out);
bool fv_kernel_f64(int dim, int rs, bool mhd, int scheme, FVKernelInfo* out);
// the split and VAN_ALBADA_PP instantiations (own translation units)
bool fv_kernel_f32_schemes(int dim, int rs, bool mhd, int scheme, FVKernelInfo* out);
bool fv_kernel_f64_schemes(int dim, int rs, bool mhd, int scheme, FVKernelInfo* out);
// the split sweeps with the AM_HLLC / HYBRID_HLLC switch (family 4)
bool fv_kernel_f32_split_am(int dim, bool mhd, FVKernelInfo* out);
bool fv_kernel_f64_split_am(int dim, bool mhd, FVKernelInfo* out);

}  // namespace amx
