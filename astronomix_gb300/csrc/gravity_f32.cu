// FP32 gravitational source-term kernels, compiled with approximate division
// and square root like the other FP32 finite-volume units (held to the FP32
// tolerance against the FP64 oracle).
#include "gravity_source.cuh"

namespace amx {
template int grav_source_launch<float>(const GravSrc<float>&, int, int, cudaStream_t);
}  // namespace amx
