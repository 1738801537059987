// Device build of the reference's advection_step.cu (TEST AND MEASUREMENT INFRASTRUCTURE ONLY).
#include "gpu_shim.cuh"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
namespace ref_adv {
#include "4_0_Calculus_ToolBox/advection_step.cu"
}
#pragma pop_macro("__global__")

VSL_REF_KERNEL void vslref_advection_step(double *astep, const double *vx, const double *vy, const double *vz,
                    const double *lsf, int rows, int cols, int pges, double dx, double dy, double dz)
{
    ref_adv::advection_step(astep, vx, vy, vz, lsf, rows, cols, pges, dx, dy, dz);
}
