// Host build of one reference WENO5 extension kernel file (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_un5 {
VSL_REF_MATH
#include "2_2_WENO5RK3_Extend/upwind_normal.cu"
}

extern "C" void ref_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                                  const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                                  const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                                  int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_un5::upwind_normal(nx, ny, nz, lsf, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz,
                                          num_ele));
}
