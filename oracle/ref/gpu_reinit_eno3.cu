// Device build of the reference's weno_rk3_reinitialization.cu (TEST AND MEASUREMENT INFRASTRUCTURE ONLY).
#include "gpu_shim.cuh"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
namespace ref_re3 {
#include "1_1_WENORK3_Reinitialization/weno_rk3_reinitialization.cu"
}
#pragma pop_macro("__global__")

VSL_REF_KERNEL void vslref_cubic_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu,
                    double *zpd, const double *lsf, int num_ele, int rows, int cols, int pges, double dx, double dy,
                    double dz)
{
    ref_re3::boundary_correction(xpr, xpl, ypf, ypb, zpu, zpd, lsf, num_ele, rows, cols, pges, dx, dy, dz);
}

VSL_REF_KERNEL void vslref_re_step_eno3(double *step, const double *lsf, const bool *mask, const double *deltat,
                    const double *xpr, const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                    const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz, int num_ele)
{
    ref_re3::re_step(step, lsf, mask, deltat, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz, num_ele);
}
