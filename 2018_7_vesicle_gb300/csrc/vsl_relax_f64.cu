// vsl_relax_f64.cu -- FP64 instantiation of the relaxation-step kernels (vsl_relax.cuh),
// compiled without multiply-add contraction, and the 2x2 tension/pressure solve.
#include "vsl_relax.cuh"

namespace vsl {

VSL_INSTANTIATE_RELAX(double)

cudaError_t launch_tension_pressure(const double *moments, const double *area_volume, const double *dt, double A0,
                                    double V0, double *tp, cudaStream_t s)
{
    k_tension_pressure<<<1, 32, 0, s>>>(moments, area_volume, dt, A0, V0, tp);
    return cudaGetLastError();
}

}  // namespace vsl
