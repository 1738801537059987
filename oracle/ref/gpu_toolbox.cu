// Device build of the reference's set_calculus_toolbox.cu (TEST AND MEASUREMENT INFRASTRUCTURE ONLY).
#include "gpu_shim.cuh"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
namespace ref_ct {
#include "4_0_Calculus_ToolBox/set_calculus_toolbox.cu"
}
#pragma pop_macro("__global__")

VSL_REF_KERNEL void vslref_set_calculus_toolbox(double *Fx, double *Fy, double *Fz, double *FGradMag, double *Nx,
                    double *Ny, double *Nz, double *Fxx, double *Fyy, double *Fzz, double *Fxy, double *Fyz,
                    double *Fzx, double *FLaplacian, double *MeanCurvature, double *GaussianCurvature,
                    double *Heaviside, double *DiracDelta, const double *lsf, const double *HPrimal, int rows,
                    int cols, int pges, double dx, double dy, double dz, double ds, int num_ele)
{
    ref_ct::set_calculus_toolbox(Fx, Fy, Fz, FGradMag, Nx, Ny, Nz, Fxx, Fyy, Fzz, Fxy, Fyz, Fzx, FLaplacian,
        MeanCurvature, GaussianCurvature, Heaviside, DiracDelta, lsf, HPrimal, rows, cols, pges, dx, dy, dz, ds,
        num_ele);
}
