// Batched FV kernel instantiations for float state arrays.
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

bool fv_batch_kernel_f32(int dim, int rs, bool mhd, int variant, BatchKernelInfo* out) {
  AMX_BATCH_CASE(2, RS_HLL, false, 0)
  AMX_BATCH_CASE(2, RS_HLL, true, 0)
  AMX_BATCH_CASE(2, RS_HLLC, false, 0)
  AMX_BATCH_CASE(2, RS_HLLC, true, 0)
  return fv_batch_kernel_f32_alt(dim, rs, mhd, variant, out);
}

}  // namespace amx
