// Device build of the reference's re_step.cu (TEST AND MEASUREMENT INFRASTRUCTURE ONLY).
#include "gpu_shim.cuh"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
namespace ref_re5 {
#include "1_3_WENO5RK3_Reinitialization/re_step.cu"
}
#pragma pop_macro("__global__")

VSL_REF_KERNEL void vslref_re_step(double *step, const double *lsf, const bool *mask, const double *deltat,
                    const double *xpr, const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                    const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz, int num_ele)
{
    ref_re5::re_step(step, lsf, mask, deltat, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz, num_ele);
}
