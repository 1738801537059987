// Host build of one reference WENO5 extension kernel file (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_bi5 {
VSL_REF_MATH
#include "2_2_WENO5RK3_Extend/boundary_interpolant.cu"
}

extern "C" void ref_boundary_interpolant(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu,
                                         double *cpd, const double *xpr, const double *xpl, const double *ypf,
                                         const double *ypb, const double *zpu, const double *zpd, const double *lsf,
                                         int rows, int cols, int pges, double dx, double dy, double dz, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_bi5::boundary_interpolant(cpr, cpl, cpf, cpb, cpu, cpd, xpr, xpl, ypf, ypb, zpu, zpd, lsf, rows,
                                                 cols, pges, dx, dy, dz, num_ele));
}
