// vsl_fused_f32.cu -- instantiation of the fused stage kernels for float.
// FP32 mixed-precision form (stencils in FP32, interface roots in FP64).
#include "vsl_fused.cuh"
#include "vsl_tiled.cuh"

namespace vsl {
VSL_INSTANTIATE_FUSED(float)
}  // namespace vsl
