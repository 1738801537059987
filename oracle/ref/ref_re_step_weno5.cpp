// Host build of the reference WENO5 re_step kernel (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_re5 {
VSL_REF_MATH
#include "1_3_WENO5RK3_Reinitialization/re_step.cu"
}

extern "C" void ref_re_step(double *step, const double *lsf, const bool *mask, const double *deltat,
                            const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                            const double *zpu, const double *zpd, int rows, int cols, int pges, double dx,
                            double dy, double dz, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_re5::re_step(step, lsf, mask, deltat, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy,
                                    dz, num_ele));
}
