// Device build of the reference's boundary_interpolant.cu (TEST AND MEASUREMENT INFRASTRUCTURE ONLY).
#include "gpu_shim.cuh"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
namespace ref_bi5 {
#include "2_2_WENO5RK3_Extend/boundary_interpolant.cu"
}
#pragma pop_macro("__global__")

VSL_REF_KERNEL void vslref_boundary_interpolant(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu,
                    double *cpd, const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                    const double *zpu, const double *zpd, const double *lsf, int rows, int cols, int pges, double dx,
                    double dy, double dz, int num_ele)
{
    ref_bi5::boundary_interpolant(cpr, cpl, cpf, cpb, cpu, cpd, xpr, xpl, ypf, ypb, zpu, zpd, lsf, rows, cols, pges,
        dx, dy, dz, num_ele);
}
