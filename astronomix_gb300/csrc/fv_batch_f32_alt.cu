// Batched FV kernel instantiations for float state arrays (alternative tile shapes).
#include "fv_batch.cuh"
#include "fv_batch_registry.h"

namespace amx {

#define AMX_BATCH_CASE(D, R, M, V)                              \
  if (dim == D && rs == R && mhd == M && variant == V) {        \
    out->fn = (const void*)&fv_batch_kernel<float, D, R, M, V>; \
    out->smem = TileGeom<float, D, V>::SMEM;                    \
    out->variant = V;                                           \
    out->tile0 = TileGeom<float, D, V>::T0;                     \
    out->tile1 = TileGeom<float, D, V>::T1;                     \
    return true;                                                \
  }

bool fv_batch_kernel_f32_alt(int dim, int rs, bool mhd, int variant, BatchKernelInfo* out) {
  AMX_BATCH_CASE(2, RS_HLL, false, 1)
  AMX_BATCH_CASE(2, RS_HLL, true, 1)
  AMX_BATCH_CASE(2, RS_HLLC, false, 1)
  AMX_BATCH_CASE(2, RS_HLLC, true, 1)
  AMX_BATCH_CASE(2, RS_HLL, false, 2)
  AMX_BATCH_CASE(2, RS_HLL, true, 2)
  AMX_BATCH_CASE(2, RS_HLLC, false, 2)
  AMX_BATCH_CASE(2, RS_HLLC, true, 2)
  return false;
}

}  // namespace amx
