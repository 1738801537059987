/*
 * vsl_oracle.h -- CPU restatement of the level-set hot path (TEST INFRASTRUCTURE ONLY).
 *
 * One function per reference kernel, same argument order as the reference prototype,
 * host pointers, FP64.  Only tests/, the smoke check and the bench's CPU-baseline leg use
 * this library; the product never links it.
 */
#ifndef VSL_ORACLE_H
#define VSL_ORACLE_H

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

void orc_boundary_location(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                           const double *lsf, int num_ele, int rows, int cols, int pges, double dx, double dy,
                           double dz);
void orc_cubic_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                                   const double *lsf, int num_ele, int rows, int cols, int pges, double dx,
                                   double dy, double dz);
void orc_re_step(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                 const double *xpl, const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                 int rows, int cols, int pges, double dx, double dy, double dz, int num_ele);
void orc_re_step_eno3(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                      const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                      const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                      int num_ele);
void orc_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr, const double *xpl,
                       const double *ypf, const double *ypb, const double *zpu, const double *zpd, int rows,
                       int cols, int pges, double dx, double dy, double dz, int num_ele);
void orc_upwind_normal_eno3(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                            const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                            const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                            int num_ele);
void orc_boundary_interpolant(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                              const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                              const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                              int pges, double dx, double dy, double dz, int num_ele);
void orc_boundary_interpolate_eno3(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                                   const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                   const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                                   int pges, double dx, double dy, double dz, int num_ele);
void orc_extend_step(double *step, const double *deltat, const double *lsf, const double *vx, const double *vy,
                     const double *vz, const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                     const double *zpu, const double *zpd, const double *cpr, const double *cpl,
                     const double *cpf, const double *cpb, const double *cpu, const double *cpd, int rows,
                     int cols, int pges, double dx, double dy, double dz, int num_ele);
void orc_extend_step_eno3(double *step, const double *deltat, const double *lsf, const double *vx,
                          const double *vy, const double *vz, const double *xpr, const double *xpl,
                          const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                          const double *cpr, const double *cpl, const double *cpf, const double *cpb,
                          const double *cpu, const double *cpd, int rows, int cols, int pges, double dx, double dy,
                          double dz, int num_ele);
void orc_advection_step(double *astep, const double *vx, const double *vy, const double *vz, const double *lsf,
                        int rows, int cols, int pges, double dx, double dy, double dz);
void orc_weno_derivative(double *back_x, double *fore_x, double *back_y, double *fore_y, double *back_z,
                         double *fore_z, const double *lsf, int rows, int cols, int pges, double dx, double dy,
                         double dz);
void orc_set_calculus_toolbox(double *Fx, double *Fy, double *Fz, double *FGradMag, double *Nx, double *Ny,
                              double *Nz, double *Fxx, double *Fyy, double *Fzz, double *Fxy, double *Fyz,
                              double *Fzx, double *FLaplacian, double *MeanCurvature, double *GaussianCurvature,
                              double *Heaviside, double *DiracDelta, const double *lsf, const double *HPrimal,
                              int rows, int cols, int pges, double dx, double dy, double dz, double ds, int num_ele);
void orc_auxi_set_calculus_toolbox(
    double *Ax, double *Ay, double *Az, double *AGradMag, double *ACx, double *ACy, double *ACz,
    double *ANormCrossAF, double *Tx, double *Ty, double *Tz, double *Anx, double *Any, double *Anz, double *Axx,
    double *Ayy, double *Azz, double *Axy, double *Ayz, double *Azx, double *ALaplacian, double *GeodesicCurvature,
    double *NormalCurvature, double *GeodesicTorsion, double *BPerpendicular, double *AHeaviside,
    double *ADiracDelta, const double *lsf, const double *AHPrimal, const double *Fx, const double *Fy,
    const double *Fz, const double *FGradMag, const double *Nx, const double *Ny, const double *Nz,
    const double *Fxx, const double *Fyy, const double *Fzz, const double *Fxy, const double *Fyz,
    const double *Fzx, int rows, int cols, int pges, double dx, double dy, double dz, double ds, int num_ele);
void orc_enork2_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                                    const double *lsf, int num_ele, int rows, int cols, int pges, double dx,
                                    double dy, double dz);
void orc_enork2_re_step(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                        const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                        const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                        int num_ele);
void orc_enork2_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                              const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                              const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                              int num_ele);
void orc_enork2_boundary_interpolate(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                                     const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                     const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                                     int pges, double dx, double dy, double dz, int num_ele);
void orc_enork2_extend_step(double *step, const double *deltat, const double *lsf, const double *vx,
                            const double *vy, const double *vz, const double *xpr, const double *xpl,
                            const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                            const double *cpr, const double *cpl, const double *cpf, const double *cpb,
                            const double *cpu, const double *cpd, int rows, int cols, int pges, double dx, double dy,
                            double dz, int num_ele);
int orc_version(void);

#ifdef __cplusplus
}
#endif

#endif
