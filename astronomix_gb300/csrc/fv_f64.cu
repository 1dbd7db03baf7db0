// FV kernel instantiations for double state arrays.
#include "fv_kernels.cuh"
#include "fv_registry.h"

namespace amx {

#define AMX_FV_CASE(D, R, M)                                                  \
  if (dim == D && rs == R && mhd == M) {                                      \
    out->fn = (const void*)&fv_run_kernel<double, D, R, M, FV_UNSPLIT>;                    \
    out->smem = TileGeom<double, D>::SMEM;                                     \
    out->smem_pp = TileGeom<double, D>::PP_SMEM;                               \
    return true;                                                              \
  }

bool fv_kernel_f64(int dim, int rs, bool mhd, int scheme, FVKernelInfo* out) {
  if (scheme != FV_UNSPLIT) return fv_kernel_f64_schemes(dim, rs, mhd, scheme, out);
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
  // AM_HLLC / HYBRID_HLLC (unsplit only)
  AMX_FV_CASE(1, RS_AM, false)
  AMX_FV_CASE(2, RS_AM, false)
  AMX_FV_CASE(2, RS_AM, true)
  AMX_FV_CASE(3, RS_AM, false)
  AMX_FV_CASE(3, RS_AM, true)
  return false;
}

}  // namespace amx
