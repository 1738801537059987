// Host build of one reference kernel file
// (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_wd {
VSL_REF_MATH
#include "5_0_Nonoscillating_Reconstruction/nonoscillating_interpolant.cu"
}

extern "C" void ref_weno_derivative(double *bx, double *fx, double *by, double *fy, double *bz, double *fz,
                                    const double *lsf, int rows, int cols, int pges, double dx, double dy, double dz)
{
    VSL_REF_LAUNCH(rows, cols, pges, ref_wd::weno_derivative(bx, fx, by, fy, bz, fz, lsf, rows, cols, pges, dx, dy, dz));
}
