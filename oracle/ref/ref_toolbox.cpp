// Host build of one reference kernel file
// (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_ct {
VSL_REF_MATH
#include "4_0_Calculus_ToolBox/set_calculus_toolbox.cu"
}

extern "C" void ref_set_calculus_toolbox(double *Fx, double *Fy, double *Fz, double *FGradMag, double *Nx,
                                         double *Ny, double *Nz, double *Fxx, double *Fyy, double *Fzz, double *Fxy,
                                         double *Fyz, double *Fzx, double *FLaplacian, double *MeanCurvature,
                                         double *GaussianCurvature, double *Heaviside, double *DiracDelta,
                                         const double *lsf, const double *HPrimal, int rows, int cols, int pges,
                                         double dx, double dy, double dz, double ds, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_ct::set_calculus_toolbox(Fx, Fy, Fz, FGradMag, Nx, Ny, Nz, Fxx, Fyy, Fzz, Fxy, Fyz, Fzx,
                                                FLaplacian, MeanCurvature, GaussianCurvature, Heaviside, DiracDelta,
                                                lsf, HPrimal, rows, cols, pges, dx, dy, dz, ds, num_ele));
}
