// vsl_relax_f32.cu -- FP32 (mixed-form) instantiation of the relaxation-step kernels of
// vsl_relax.cuh; the surface integrals stay FP64.
#include "vsl_relax.cuh"

namespace vsl {

VSL_INSTANTIATE_RELAX(float)

}  // namespace vsl
