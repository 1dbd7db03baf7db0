// Adjoint kernels for float state arrays.
#include "adjoint_impl.cuh"

namespace amx {
namespace adj {
bool ops_f32(int dim, Ops* out) { return ops<float>(dim, out); }
}  // namespace adj
}  // namespace amx
