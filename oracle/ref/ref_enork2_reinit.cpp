// Host build of the reference ENORK2 reinitialization kernels (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_er2 {
VSL_REF_MATH
#include "1_0_ENORK2_Reinitialization/boundary_correction.cu"
}

extern "C" void ref_enork2_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu,
                                               double *zpd, const double *lsf, int num_ele, int rows, int cols,
                                               int pges, double dx, double dy, double dz)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_er2::boundary_correction(xpr, xpl, ypf, ypb, zpu, zpd, lsf, num_ele, rows, cols, pges, dx, dy,
                                                dz));
}

extern "C" void ref_enork2_re_step(double *step, const double *lsf, const bool *mask, const double *deltat,
                                   const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                   const double *zpu, const double *zpd, int rows, int cols, int pges, double dx,
                                   double dy, double dz, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_er2::re_step(step, lsf, mask, deltat, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy,
                                    dz, num_ele));
}
