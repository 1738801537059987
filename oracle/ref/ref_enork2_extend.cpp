// Host build of the reference ENORK2 extension kernels (TEST INFRASTRUCTURE ONLY).
#include "ref_shim.hpp"

namespace ref_ex2 {
VSL_REF_MATH
#include "2_0_ENORK2_Extend/enork2_extend.cu"
}

extern "C" void ref_enork2_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                                         const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                                         const double *zpd, int rows, int cols, int pges, double dx, double dy,
                                         double dz, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_ex2::upwind_normal(nx, ny, nz, lsf, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz,
                                          num_ele));
}

extern "C" void ref_enork2_boundary_interpolate(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu,
                                                double *cpd, const double *xpr, const double *xpl, const double *ypf,
                                                const double *ypb, const double *zpu, const double *zpd,
                                                const double *lsf, int rows, int cols, int pges, double dx, double dy,
                                                double dz, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_ex2::boundary_interpolate(cpr, cpl, cpf, cpb, cpu, cpd, xpr, xpl, ypf, ypb, zpu, zpd, lsf, rows,
                                                 cols, pges, dx, dy, dz, num_ele));
}

extern "C" void ref_enork2_extend_step(double *step, const double *deltat, const double *lsf, const double *vx,
                                       const double *vy, const double *vz, const double *xpr, const double *xpl,
                                       const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                                       const double *cpr, const double *cpl, const double *cpf, const double *cpb,
                                       const double *cpu, const double *cpd, int rows, int cols, int pges, double dx,
                                       double dy, double dz, int num_ele)
{
    VSL_REF_LAUNCH(rows, cols, pges,
                   ref_ex2::extend_step(step, deltat, lsf, vx, vy, vz, xpr, xpl, ypf, ypb, zpu, zpd, cpr, cpl, cpf,
                                        cpb, cpu, cpd, rows, cols, pges, dx, dy, dz, num_ele));
}
