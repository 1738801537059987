// Device build of the reference's extend_step.cu (TEST AND MEASUREMENT INFRASTRUCTURE ONLY).
#include "gpu_shim.cuh"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
namespace ref_ex5 {
#include "2_2_WENO5RK3_Extend/extend_step.cu"
}
#pragma pop_macro("__global__")

VSL_REF_KERNEL void vslref_extend_step(double *step, const double *deltat, const double *lsf, const double *vx,
                    const double *vy, const double *vz, const double *xpr, const double *xpl, const double *ypf,
                    const double *ypb, const double *zpu, const double *zpd, const double *cpr, const double *cpl,
                    const double *cpf, const double *cpb, const double *cpu, const double *cpd, int rows, int cols,
                    int pges, double dx, double dy, double dz, int num_ele)
{
    ref_ex5::extend_step(step, deltat, lsf, vx, vy, vz, xpr, xpl, ypf, ypb, zpu, zpd, cpr, cpl, cpf, cpb, cpu, cpd,
        rows, cols, pges, dx, dy, dz, num_ele);
}
