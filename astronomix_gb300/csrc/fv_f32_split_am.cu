// FV kernel instantiations for float state arrays: the split (MUSCL-Hancock)
// sweeps with the AM_HLLC / HYBRID_HLLC compression switch.  A translation
// unit of their own, compiled in parallel with the other schemes.
#include "fv_kernels.cuh"
#include "fv_registry.h"

namespace amx {

#define AMX_FV_SPLIT_AM_CASE(D, M)                                                \
  if (dim == D && mhd == M) {                                                     \
    out->fn = (const void*)&fv_run_kernel<float, D, RS_AM, M, FV_SPLIT>;           \
    out->smem = TileGeom<float, D>::SPLIT_SMEM;                                   \
    out->smem_pp = TileGeom<float, D>::PP_SMEM;                                   \
    return true;                                                                  \
  }

bool fv_kernel_f32_split_am(int dim, bool mhd, FVKernelInfo* out) {
  AMX_FV_SPLIT_AM_CASE(1, false)
  AMX_FV_SPLIT_AM_CASE(2, false)
  AMX_FV_SPLIT_AM_CASE(2, true)
  AMX_FV_SPLIT_AM_CASE(3, false)
  AMX_FV_SPLIT_AM_CASE(3, true)
  return false;
}

}  // namespace amx
