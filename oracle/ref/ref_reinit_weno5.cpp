// Host build of the reference WENO5 reinitialization kernels (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

thread_local vsl_ref_dim3 blockIdx, threadIdx, blockDim;

namespace ref_loc {
VSL_REF_MATH
#include "1_3_WENO5RK3_Reinitialization/boundary_location.cu"
}

extern "C" void ref_boundary_location(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                                      const double *lsf, int num_ele, int rows, int cols, int pges, double dx,
                                      double dy, double dz)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_loc::boundary_location(xpr, xpl, ypf, ypb, zpu, zpd, lsf, num_ele, rows, cols, pges, dx, dy, dz));
}
