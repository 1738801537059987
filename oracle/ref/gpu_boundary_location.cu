// Device build of the reference's boundary_location.cu (TEST AND MEASUREMENT INFRASTRUCTURE ONLY).
#include "gpu_shim.cuh"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
namespace ref_loc {
#include "1_3_WENO5RK3_Reinitialization/boundary_location.cu"
}
#pragma pop_macro("__global__")

VSL_REF_KERNEL void vslref_boundary_location(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu,
                    double *zpd, const double *lsf, int num_ele, int rows, int cols, int pges, double dx, double dy,
                    double dz)
{
    ref_loc::boundary_location(xpr, xpl, ypf, ypb, zpu, zpd, lsf, num_ele, rows, cols, pges, dx, dy, dz);
}
