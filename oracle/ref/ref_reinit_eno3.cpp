// Host build of the reference WENORK3 ("ENO3") reinitialization kernels (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_re3 {
VSL_REF_MATH
#include "1_1_WENORK3_Reinitialization/weno_rk3_reinitialization.cu"
}

extern "C" void ref_cubic_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu,
                                              double *zpd, const double *lsf, int num_ele, int rows, int cols,
                                              int pges, double dx, double dy, double dz)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_re3::boundary_correction(xpr, xpl, ypf, ypb, zpu, zpd, lsf, num_ele, rows, cols, pges, dx, dy,
                                                dz));
}

extern "C" void ref_re_step_eno3(double *step, const double *lsf, const bool *mask, const double *deltat,
                                 const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                 const double *zpu, const double *zpd, int rows, int cols, int pges, double dx,
                                 double dy, double dz, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_re3::re_step(step, lsf, mask, deltat, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy,
                                    dz, num_ele));
}
