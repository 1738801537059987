// vsl_auxi_f32.cu -- the FP32 (mixed-form) instantiation of the auxiliary level set
// toolbox and the masked integrals (vsl_auxi.cuh), with the FP32 form's fast division;
// the integrals are summed in FP64.
#include "vsl_auxi.cuh"

namespace vsl {

VSL_INSTANTIATE_AUXI(float)

}  // namespace vsl
