// Host build of one reference WENO5 extension kernel file (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_ex5 {
VSL_REF_MATH
#include "2_2_WENO5RK3_Extend/extend_step.cu"
}

extern "C" void ref_extend_step(double *step, const double *deltat, const double *lsf, const double *vx,
                                const double *vy, const double *vz, const double *xpr, const double *xpl,
                                const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                                const double *cpr, const double *cpl, const double *cpf, const double *cpb,
                                const double *cpu, const double *cpd, int rows, int cols, int pges, double dx,
                                double dy, double dz, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_ex5::extend_step(step, deltat, lsf, vx, vy, vz, xpr, xpl, ypf, ypb, zpu, zpd, cpr, cpl, cpf, cpb,
                                        cpu, cpd, rows, cols, pges, dx, dy, dz, num_ele));
}
