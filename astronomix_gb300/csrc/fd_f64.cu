// FD kernel instantiations for float64 states (IEEE operations).
#include "fd_impl.cuh"

namespace amx {
namespace fd {
AMX_FD_INSTANTIATE(double, f64)
}  // namespace fd
}  // namespace amx
