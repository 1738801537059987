// Host build of one reference kernel file
// (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_adv {
VSL_REF_MATH
#include "4_0_Calculus_ToolBox/advection_step.cu"
}

extern "C" void ref_advection_step(double *astep, const double *vx, const double *vy, const double *vz,
                                   const double *lsf, int rows, int cols, int pges, double dx, double dy, double dz)
{
    VSL_REF_LAUNCH(rows, cols, pges, ref_adv::advection_step(astep, vx, vy, vz, lsf, rows, cols, pges, dx, dy, dz));
}
