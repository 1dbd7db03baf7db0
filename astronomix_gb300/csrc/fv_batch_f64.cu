// Batched FV kernel instantiations for double state arrays.
#include "fv_batch.cuh"
#include "fv_batch_registry.h"

namespace amx {

#define AMX_BATCH_CASE(D, R, M, V)                              \
  if (dim == D && rs == R && mhd == M && variant == V) {        \
    out->fn = (const void*)&fv_batch_kernel<double, D, R, M, V>; \
    out->smem = TileGeom<double, D, V>::SMEM;                    \
    out->variant = V;                                           \
    out->tile0 = TileGeom<double, D, V>::T0;                     \
    out->tile1 = TileGeom<double, D, V>::T1;                     \
    return true;                                                \
  }

bool fv_batch_kernel_f64(int dim, int rs, bool mhd, int variant, BatchKernelInfo* out) {
  AMX_BATCH_CASE(2, RS_HLL, false, 0)
  AMX_BATCH_CASE(2, RS_HLL, true, 0)
  AMX_BATCH_CASE(2, RS_HLLC, false, 0)
  AMX_BATCH_CASE(2, RS_HLLC, true, 0)
  return false;
}

}  // namespace amx
