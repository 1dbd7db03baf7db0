// FV kernel instantiations for double state arrays.
#include "fv_kernels.cuh"
#include "fv_registry.h"

namespace amx {

#define AMX_FV_CASE(D, R, M)                                                  \
  if (dim == D && rs == R && mhd == M) {                                      \
    out->fn = (const void*)&fv_run_kernel<double, D, R, M>;                    \
    out->smem = TileGeom<double, D>::SMEM;                                     \
    return true;                                                              \
  }

bool fv_kernel_f64(int dim, int rs, bool mhd, FVKernelInfo* out) {
  AMX_FV_CASE(1, RS_HLL, false)
  AMX_FV_CASE(1, RS_HLLC, false)
  AMX_FV_CASE(1, RS_LF, false)
  AMX_FV_CASE(2, RS_HLL, false)
  AMX_FV_CASE(2, RS_HLLC, false)
  AMX_FV_CASE(2, RS_LF, false)
  AMX_FV_CASE(2, RS_HLL, true)
  AMX_FV_CASE(2, RS_HLLC, true)
  AMX_FV_CASE(2, RS_LF, true)
  AMX_FV_CASE(3, RS_HLL, false)
  AMX_FV_CASE(3, RS_HLLC, false)
  AMX_FV_CASE(3, RS_LF, false)
  AMX_FV_CASE(3, RS_HLL, true)
  AMX_FV_CASE(3, RS_HLLC, true)
  AMX_FV_CASE(3, RS_LF, true)
  return false;
}

}  // namespace amx
