// FD kernel instantiations for float32 states (approximate div/sqrt allowed).
#include "fd_impl.cuh"

namespace amx {
namespace fd {
AMX_FD_INSTANTIATE(float, f32)
}  // namespace fd
}  // namespace amx
