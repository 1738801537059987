// vsl_fused_f64.cu -- instantiation of the fused stage kernels for double.
// FP64 plain form: built with -fmad=false, every product and sum rounded on its own as in
// the reference's FP64 kernels.
#include "vsl_fused.cuh"

namespace vsl {
VSL_INSTANTIATE_FUSED(double)

cudaError_t launch_condition_reset(cudaGraphConditionalHandle handle, cudaStream_t s)
{
    k_condition_reset<<<1, 1, 0, s>>>(handle);
    return cudaGetLastError();
}
}  // namespace vsl
