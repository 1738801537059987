// Device build of the reference's upwind_normal.cu (TEST AND MEASUREMENT INFRASTRUCTURE ONLY).
#include "gpu_shim.cuh"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
namespace ref_un5 {
#include "2_2_WENO5RK3_Extend/upwind_normal.cu"
}
#pragma pop_macro("__global__")

VSL_REF_KERNEL void vslref_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                    const double *xpl, const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                    int rows, int cols, int pges, double dx, double dy, double dz, int num_ele)
{
    ref_un5::upwind_normal(nx, ny, nz, lsf, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz, num_ele);
}
