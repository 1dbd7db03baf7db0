// Adjoint kernels for double state arrays.
#include "adjoint_impl.cuh"

namespace amx {
namespace adj {
bool ops_f64(int dim, Ops* out) { return ops<double>(dim, out); }
}  // namespace adj
}  // namespace amx
