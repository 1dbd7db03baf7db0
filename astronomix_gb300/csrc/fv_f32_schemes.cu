// FV kernel instantiations for float state arrays: the split (MUSCL-Hancock)
// and the VAN_ALBADA_PP schemes.
#include "fv_kernels.cuh"
#include "fv_registry.h"

namespace amx {

#define AMX_FV_SCHEME_CASE(D, R, M, S)                                       \
  if (dim == D && rs == R && mhd == M && scheme == S) {                      \
    out->fn = (const void*)&fv_run_kernel<float, D, R, M, S>;                 \
    out->smem = S == FV_SPLIT ? TileGeom<float, D>::SPLIT_SMEM : TileGeom<float, D>::SMEM; \
    out->smem_pp = TileGeom<float, D>::PP_SMEM;                               \
    return true;                                                             \
  }

bool fv_kernel_f32_schemes(int dim, int rs, bool mhd, int scheme, FVKernelInfo* out) {
  if (scheme == FV_SPLIT && rs == RS_AM) return fv_kernel_f32_split_am(dim, mhd, out);
  AMX_FV_SCHEME_CASE(1, RS_HLL, false, FV_SPLIT)
  AMX_FV_SCHEME_CASE(1, RS_HLLC, false, FV_SPLIT)
  AMX_FV_SCHEME_CASE(1, RS_LF, false, FV_SPLIT)
  AMX_FV_SCHEME_CASE(2, RS_HLL, false, FV_SPLIT)
  AMX_FV_SCHEME_CASE(2, RS_HLLC, false, FV_SPLIT)
  AMX_FV_SCHEME_CASE(2, RS_LF, false, FV_SPLIT)
  AMX_FV_SCHEME_CASE(2, RS_HLL, true, FV_SPLIT)
  AMX_FV_SCHEME_CASE(2, RS_HLLC, true, FV_SPLIT)
  AMX_FV_SCHEME_CASE(2, RS_LF, true, FV_SPLIT)
  AMX_FV_SCHEME_CASE(3, RS_HLL, false, FV_SPLIT)
  AMX_FV_SCHEME_CASE(3, RS_HLLC, false, FV_SPLIT)
  AMX_FV_SCHEME_CASE(3, RS_LF, false, FV_SPLIT)
  AMX_FV_SCHEME_CASE(3, RS_HLL, true, FV_SPLIT)
  AMX_FV_SCHEME_CASE(3, RS_HLLC, true, FV_SPLIT)
  AMX_FV_SCHEME_CASE(3, RS_LF, true, FV_SPLIT)
  AMX_FV_SCHEME_CASE(2, RS_HLL, false, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(2, RS_HLLC, false, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(2, RS_LF, false, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(2, RS_HLL, true, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(2, RS_HLLC, true, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(2, RS_LF, true, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(3, RS_HLL, false, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(3, RS_HLLC, false, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(3, RS_LF, false, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(3, RS_HLL, true, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(3, RS_HLLC, true, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(3, RS_LF, true, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(2, RS_AM, false, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(2, RS_AM, true, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(3, RS_AM, false, FV_UNSPLIT_PP)
  AMX_FV_SCHEME_CASE(3, RS_AM, true, FV_UNSPLIT_PP)
  return false;
}

}  // namespace amx
