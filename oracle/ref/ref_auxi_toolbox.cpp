// Host build of one reference kernel file
// (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_at {
VSL_REF_MATH
#include "4_0_Calculus_ToolBox/auxi_set_calculus_toolbox.cu"
}

extern "C" void ref_auxi_set_calculus_toolbox(
    double *Ax, double *Ay, double *Az, double *AGradMag, double *ACx, double *ACy, double *ACz,
    double *ANormCrossAF, double *Tx, double *Ty, double *Tz, double *Anx, double *Any, double *Anz, double *Axx,
    double *Ayy, double *Azz, double *Axy, double *Ayz, double *Azx, double *ALaplacian, double *GeodesicCurvature,
    double *NormalCurvature, double *GeodesicTorsion, double *BPerpendicular, double *AHeaviside,
    double *ADiracDelta, const double *lsf, const double *AHPrimal, const double *Fx, const double *Fy,
    const double *Fz, const double *FGradMag, const double *Nx, const double *Ny, const double *Nz,
    const double *Fxx, const double *Fyy, const double *Fzz, const double *Fxy, const double *Fyz,
    const double *Fzx, int rows, int cols, int pges, double dx, double dy, double dz, double ds, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_at::auxi_set_calculus_toolbox(
                       Ax, Ay, Az, AGradMag, ACx, ACy, ACz, ANormCrossAF, Tx, Ty, Tz, Anx, Any, Anz, Axx, Ayy, Azz,
                       Axy, Ayz, Azx, ALaplacian, GeodesicCurvature, NormalCurvature, GeodesicTorsion,
                       BPerpendicular, AHeaviside, ADiracDelta, lsf, AHPrimal, Fx, Fy, Fz, FGradMag, Nx, Ny, Nz, Fxx,
                       Fyy, Fzz, Fxy, Fyz, Fzx, rows, cols, pges, dx, dy, dz, ds, num_ele));
}
