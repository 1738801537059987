// vsl_toolbox_f32.cu -- the FP32 (mixed-form) instantiation of the toolbox and
// band-maximum kernels of vsl_toolbox.cuh, compiled with the FP32 form's fast division.
#include "vsl_toolbox.cuh"

namespace vsl {

template cudaError_t launch_toolbox<float>(const float *, ToolboxOut<float>, const Grid &, double, double *, int *,
                                           cudaStream_t);
template cudaError_t launch_band_maxabs<float>(const float *, const float *, double, const Grid &, double *, int *,
                                               cudaStream_t);

}  // namespace vsl
