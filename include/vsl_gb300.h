/*
 * vsl_gb300.h -- C ABI of the GB300 level-set hot path (vesicle code).
 *
 * Layout of every field (the reference's MATLAB gpuArray layout): a rows x cols x pges
 * column-major array, element (i, j, k) at k*rows*cols + j*rows + i, with i = row (y),
 * j = column (x), k = page (z); dx is the column spacing, dy the row spacing, dz the page
 * spacing.  Neighbours outside the grid are clamped to the edge.
 *
 * All pointers are DEVICE pointers on the current CUDA device, the work is enqueued on
 * `stream` (NULL = legacy default stream) and the call returns once it is enqueued.  No
 * entry point allocates memory: callers pass outputs and, for the composite operations,
 * a workspace of at least vsl_workspace_bytes(...) bytes (256-byte aligned).
 *
 * Return value: VSL_OK or one of the VSL_ERR_* codes below.
 *
 * Citations "ref: file:line" name the reference function each entry point replaces,
 * relative to src/7_0_paper/2_0_Vesicle/ of tiankuizhang/2018_7_Vesicle.
 */
#ifndef VSL_GB300_H
#define VSL_GB300_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *vsl_stream_t; /* same type as cudaStream_t */

enum {
    VSL_OK = 0,
    VSL_ERR_NULL = 1,      /* a required pointer is NULL */
    VSL_ERR_SHAPE = 2,     /* rows/cols/pges not positive, too large, or != num_ele */
    VSL_ERR_VALUE = 3,     /* a spacing, iteration count or CFL number out of range */
    VSL_ERR_WORKSPACE = 4, /* workspace missing, too small or misaligned */
    VSL_ERR_CUDA = 5,      /* a kernel launch failed (cudaGetLastError) */
    VSL_ERR_OP = 6,        /* unknown operation id */
    VSL_ERR_SCRATCH_LIMIT = 7 /* grid needs more than the static scratch of a no-allocation entry point */
};

/* largest grid accepted (nodes); indices are 64-bit inside the kernels */
#define VSL_MAX_NODES 2147483647LL

const char *vsl_status_string(int status);
int vsl_version(void);

/* ===================================================================================== */
/* Drop-in kernels: FP64, the reference kernel's argument order, MATLAB in/out semantics */
/* (non-const pointers are in/out; entries a kernel does not write keep their values).   */
/* ===================================================================================== */

/* ref: CUDA_Code/1_3_WENO5RK3_Reinitialization/boundary_location.cu:84-132 (boundary_location) */
int vsl_boundary_location(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                          const double *lsf, int num_ele, int rows, int cols, int pges, double dx, double dy,
                          double dz, vsl_stream_t stream);

/* ref: CUDA_Code/1_1_WENORK3_Reinitialization/weno_rk3_reinitialization.cu:251-293 (boundary_correction) */
int vsl_cubic_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                                  const double *lsf, int num_ele, int rows, int cols, int pges, double dx,
                                  double dy, double dz, vsl_stream_t stream);

/* ref: CUDA_Code/1_3_WENO5RK3_Reinitialization/re_step.cu:283-393 (re_step) */
int vsl_re_step(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                const double *xpl, const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                int rows, int cols, int pges, double dx, double dy, double dz, int num_ele, vsl_stream_t stream);

/* ref: CUDA_Code/1_1_WENORK3_Reinitialization/weno_rk3_reinitialization.cu:295-406 (re_step) */
int vsl_re_step_eno3(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                     const double *xpl, const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                     int rows, int cols, int pges, double dx, double dy, double dz, int num_ele,
                     vsl_stream_t stream);

/* ref: CUDA_Code/2_2_WENO5RK3_Extend/upwind_normal.cu:14-104 (upwind_normal) */
int vsl_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr, const double *xpl,
                      const double *ypf, const double *ypb, const double *zpu, const double *zpd, int rows, int cols,
                      int pges, double dx, double dy, double dz, int num_ele, vsl_stream_t stream);

/* ref: CUDA_Code/2_1_WENORK3_Extend/wenork3_extend.cu:202-292 (upwind_normal) */
int vsl_upwind_normal_eno3(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                           const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                           const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                           int num_ele, vsl_stream_t stream);

/* ref: CUDA_Code/2_2_WENO5RK3_Extend/boundary_interpolant.cu:102-141 (boundary_interpolant) */
int vsl_boundary_interpolant(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                             const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                             const double *zpu, const double *zpd, const double *lsf, int rows, int cols, int pges,
                             double dx, double dy, double dz, int num_ele, vsl_stream_t stream);

/* ref: CUDA_Code/2_1_WENORK3_Extend/wenork3_extend.cu:331-365 (boundary_interpolate) */
int vsl_boundary_interpolate_eno3(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                                  const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                  const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                                  int pges, double dx, double dy, double dz, int num_ele, vsl_stream_t stream);

/* ref: CUDA_Code/2_2_WENO5RK3_Extend/extend_step.cu:10-125 (extend_step) */
int vsl_extend_step(double *step, const double *deltat, const double *lsf, const double *vx, const double *vy,
                    const double *vz, const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                    const double *zpu, const double *zpd, const double *cpr, const double *cpl, const double *cpf,
                    const double *cpb, const double *cpu, const double *cpd, int rows, int cols, int pges,
                    double dx, double dy, double dz, int num_ele, vsl_stream_t stream);

/* ref: CUDA_Code/2_1_WENORK3_Extend/wenork3_extend.cu:372-487 (extend_step) */
int vsl_extend_step_eno3(double *step, const double *deltat, const double *lsf, const double *vx, const double *vy,
                         const double *vz, const double *xpr, const double *xpl, const double *ypf,
                         const double *ypb, const double *zpu, const double *zpd, const double *cpr,
                         const double *cpl, const double *cpf, const double *cpb, const double *cpu,
                         const double *cpd, int rows, int cols, int pges, double dx, double dy, double dz,
                         int num_ele, vsl_stream_t stream);

/* ---- ENORK2: second-order ENO with the sub-cell fix (Min 2010), Heun RK2 -----------
 * The kernels of CUDA_Code/1_0_ENORK2_Reinitialization/boundary_correction.cu and
 * CUDA_Code/2_0_ENORK2_Extend/enork2_extend.cu (the MATLAB objects ENORK2_*), FP64. */

/* ref: boundary_correction.cu:104 (boundary_correction).  Quadratic-ENO distance at every
 * crossed edge; entries without a crossing keep the caller's value (pre-fill with the
 * spacing, as ENORK2Reinitialization.m:10-15 does). */
int vsl_enork2_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                                   const double *lsf, int num_ele, int rows, int cols, int pges, double dx,
                                   double dy, double dz, vsl_stream_t stream);
/* ref: boundary_correction.cu:148 (re_step).  No fixed-node test. */
int vsl_enork2_re_step(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                       const double *xpl, const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                       int rows, int cols, int pges, double dx, double dy, double dz, int num_ele,
                       vsl_stream_t stream);
/* ref: enork2_extend.cu:103 (upwind_normal). */
int vsl_enork2_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                             const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                             const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                             int num_ele, vsl_stream_t stream);
/* ref: enork2_extend.cu:175 (boundary_interpolate).  Every entry is written (0 where the
 * cell is not cut). */
int vsl_enork2_boundary_interpolate(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                                    const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                    const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                                    int pges, double dx, double dy, double dz, int num_ele, vsl_stream_t stream);
/* ref: enork2_extend.cu:214 (extend_step).  No fixed-node test. */
int vsl_enork2_extend_step(double *step, const double *deltat, const double *lsf, const double *vx, const double *vy,
                           const double *vz, const double *xpr, const double *xpl, const double *ypf,
                           const double *ypb, const double *zpu, const double *zpd, const double *cpr,
                           const double *cpl, const double *cpf, const double *cpb, const double *cpu,
                           const double *cpd, int rows, int cols, int pges, double dx, double dy, double dz,
                           int num_ele, vsl_stream_t stream);

/* ref: CUDA_Code/4_0_Calculus_ToolBox/set_calculus_toolbox.cu:9-107 (set_calculus_toolbox) */
int vsl_set_calculus_toolbox(double *Fx, double *Fy, double *Fz, double *FGradMag, double *Nx, double *Ny,
                             double *Nz, double *Fxx, double *Fyy, double *Fzz, double *Fxy, double *Fyz,
                             double *Fzx, double *FLaplacian, double *MeanCurvature, double *GaussianCurvature,
                             double *Heaviside, double *DiracDelta, const double *lsf, const double *HPrimal,
                             int rows, int cols, int pges, double dx, double dy, double dz, double ds, int num_ele,
                             vsl_stream_t stream);

/* ref: CUDA_Code/4_0_Calculus_ToolBox/advection_step.cu:30-56 (advection_step) */
int vsl_advection_step(double *astep, const double *vx, const double *vy, const double *vz, const double *lsf,
                       int rows, int cols, int pges, double dx, double dy, double dz, vsl_stream_t stream);

/* ref: CUDA_Code/5_0_Nonoscillating_Reconstruction/nonoscillating_interpolant.cu:59-122 (weno_derivative) */
int vsl_weno_derivative(double *WENO_back_x, double *WENO_fore_x, double *WENO_back_y, double *WENO_fore_y,
                        double *WENO_back_z, double *WENO_fore_z, const double *lsf, int rows, int cols, int pges,
                        double dx, double dy, double dz, vsl_stream_t stream);

/* ===================================================================================== */
/* Method-level operations of the level-set object (SD.SDF3), fused GB300 kernels.        */
/* _f64: the plain form, FP64 throughout.  _f32: the mixed-precision form, FP32 fields    */
/* and stencils with the sub-cell interface roots and all reductions in FP64.             */
/* ===================================================================================== */

/* workspace operation ids for vsl_workspace_bytes */
enum {
    VSL_OP_REINIT_WENO5 = 1,
    VSL_OP_REINIT_ENO3 = 2,
    VSL_OP_EXTEND_WENO5 = 3,
    VSL_OP_EXTEND_ENO3 = 4,
    VSL_OP_SURFACE_REDISTANCE = 5,
    VSL_OP_AREA_VOLUME = 6,
    VSL_OP_ADVECTION = 7,
    VSL_OP_VESICLE_STEP = 8,
    VSL_OP_SET_DISTANCE = 9,
    VSL_OP_ADVECTION_ADJOINT = 10,
    VSL_OP_REINIT_ADJOINT = 11,
    VSL_OP_REINIT_ENORK2 = 12,
    VSL_OP_EXTEND_ENORK2 = 13,
    VSL_OP_SURFACE_REDISTANCE_ENORK2 = 14,
    VSL_OP_SMOOTH = 15,
    VSL_OP_RELAX_STEP = 16,
    VSL_OP_AUX_TOOLBOX = 17,
    VSL_OP_MASKED_INTEGRAL = 18,
    VSL_OP_REINIT_TOL = 19,
    VSL_OP_SURFACE_REDISTANCE_ENO3 = 20
};

/* Tuning of the FP32 tiled stage kernels (no counterpart in the reference).  Each block
 * marches `pages` pages of the grid; the library keeps a table of pages per (rows, cols,
 * pges, kind), kind 0 reinitialization, 1 extension, 2 advection, 3 ENORK2 extension, 4
 * ENORK2 reinitialization, used by every later launch of that shape (a CUDA graph keeps the
 * value it was recorded with).
 * Shapes not in the table use 20.  vsl_set_tile_pages(..., pages = 0) removes an entry; it returns
 * VSL_ERR_SHAPE / VSL_ERR_VALUE for a bad shape, kind or pages (1..65535), or a full
 * table (512 entries).  vsl_tile_pages returns the value in effect (0 for bad input). */
int vsl_set_tile_pages(int rows, int cols, int pges, int kind, int pages);
int vsl_tile_pages(int rows, int cols, int pges, int kind);

/* Plane loads of the FP32 tiled stage kernels (no counterpart in the reference), process-wide:
 * mode 0 (the default) loads every plane through registers; mode 1 loads them by TMA tensor
 * copies (grids with rows a multiple of 4 and 16-byte aligned fields; other grids keep the
 * register loads).  The planes are the same; the two kernels are compiled apart and fuse
 * multiply-adds differently, so results agree to a few ulp, not bit for bit (mode 0 is the
 * one the bitwise tests pin; mode 1 measured slower on GB300).  A launch takes the mode in
 * effect when it is issued (a CUDA graph keeps it).  vsl_set_plane_loads
 * returns VSL_ERR_VALUE for another mode; vsl_plane_loads returns the mode in effect.
 * vsl_tma_wait_timeouts reads how many bounded waits for a tensor copy have given up since
 * the library was loaded (0 unless a copy failed to complete; the kernel then goes on,
 * every access in bounds, with the plane's earlier contents). */
int vsl_set_plane_loads(int mode);
int vsl_plane_loads(void);
int vsl_tma_wait_timeouts(unsigned *count);

/* Bytes of workspace operation `op` needs on a rows x cols x pges grid of elements of
 * `elem_bytes` (8 for _f64, 4 for _f32); 0 for an unknown op or bad shape. */
size_t vsl_workspace_bytes(int op, int rows, int cols, int pges, int elem_bytes);

/* ref: +SD/@SDF3/setDistance.m:3-33.  Writes all six distance fields (Delta where no
 * interface crosses the edge); the workspace holds the list of crossed edges. */
int vsl_set_distance_f64(const double *F, double *xpr, double *xpl, double *ypf, double *ypb, double *zpu,
                         double *zpd, int rows, int cols, int pges, double dx, double dy, double dz, void *workspace,
                         size_t workspace_bytes, vsl_stream_t stream);
int vsl_set_distance_f32(const float *F, float *xpr, float *xpl, float *ypf, float *ypb, float *zpu, float *zpd,
                         int rows, int cols, int pges, double dx, double dy, double dz, void *workspace,
                         size_t workspace_bytes, vsl_stream_t stream);

/* ref: +SD/@SDF3/WENO5RK3Reinitialization.m:3-43.  F is advanced in place `iteration`
 * TVD-RK3 pseudo-steps with the cached distances of setDistance (mask = F<0 at entry,
 * dt = 0.3 * min distance). */
int vsl_weno5_rk3_reinitialization_f64(double *F, int iteration, const double *xpr, const double *xpl,
                                       const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                                       int rows, int cols, int pges, double dx, double dy, double dz,
                                       void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_weno5_rk3_reinitialization_f32(float *F, int iteration, const float *xpr, const float *xpl,
                                       const float *ypf, const float *ypb, const float *zpu, const float *zpd,
                                       int rows, int cols, int pges, double dx, double dy, double dz,
                                       void *workspace, size_t workspace_bytes, vsl_stream_t stream);

/* The reinitialization of vsl_weno5_rk3_reinitialization_* run until its residual is small
 * (no counterpart in the reference, whose loop runs a fixed count,
 * +SD/@SDF3/WENO5RK3Reinitialization.m:15; the fixed-count entry point above stays the
 * drop-in).  The residual is the FP64 maximum, over the nodes with |F| < band that are not
 * fixed, of | |grad F|_G - 1 |, with the Godunov norm and stencil choice of the
 * pseudo-step.  Pseudo-steps run while the residual exceeds tol and fewer than max_iters
 * were taken; the test runs on the device (a CUDA graph with a conditional loop node), so
 * the call neither waits nor reads back.  Results on the device: status[0] = pseudo-steps
 * taken, status[1] = 1 if the last residual is <= tol (0: stopped by max_iters; a NaN
 * residual never converges); residual[n] (optional, max_iters + 1 doubles) = the residual
 * after n pseudo-steps, residual[0] that of the input.  Each call records and instantiates a
 * small graph (driver resources, no device-memory allocation of its own); called while the
 * caller's stream is being captured, it adds its nodes to the caller's graph instead.
 * VSL_ERR_VALUE for max_iters < 0, tol < 0 or band <= 0.  Workspace op VSL_OP_REINIT_TOL. */
int vsl_weno5_rk3_reinitialization_tol_f64(double *F, int max_iters, double tol, double band, const double *xpr,
                                           const double *xpl, const double *ypf, const double *ypb,
                                           const double *zpu, const double *zpd, int rows, int cols, int pges,
                                           double dx, double dy, double dz, int *status, double *residual,
                                           void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_weno5_rk3_reinitialization_tol_f32(float *F, int max_iters, double tol, double band, const float *xpr,
                                           const float *xpl, const float *ypf, const float *ypb, const float *zpu,
                                           const float *zpd, int rows, int cols, int pges, double dx, double dy,
                                           double dz, int *status, double *residual, void *workspace,
                                           size_t workspace_bytes, vsl_stream_t stream);

/* ref: +SD/@SDF3/WENORK3Reinitialization.m:3-61 (cubic distances recomputed from F). */
int vsl_wenork3_reinitialization_f64(double *F, int iteration, int rows, int cols, int pges, double dx, double dy,
                                     double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_wenork3_reinitialization_f32(float *F, int iteration, int rows, int cols, int pges, double dx, double dy,
                                     double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);

/* ref: +SD/@SDF3/WENO5RK3Extend.m:9-76.  C is extended in place off the zero set of F
 * with F's cached distances. */
int vsl_weno5_rk3_extend_f64(double *C, int iteration, const double *F, const double *xpr, const double *xpl,
                             const double *ypf, const double *ypb, const double *zpu, const double *zpd, int rows,
                             int cols, int pges, double dx, double dy, double dz, void *workspace,
                             size_t workspace_bytes, vsl_stream_t stream);
int vsl_weno5_rk3_extend_f32(float *C, int iteration, const float *F, const float *xpr, const float *xpl,
                             const float *ypf, const float *ypb, const float *zpu, const float *zpd, int rows,
                             int cols, int pges, double dx, double dy, double dz, void *workspace,
                             size_t workspace_bytes, vsl_stream_t stream);

/* ref: +SD/@SDF3/WENORK3Extend.m:9-98 (cubic distances of F recomputed inside). */
int vsl_wenork3_extend_f64(double *C, int iteration, const double *F, int rows, int cols, int pges, double dx,
                           double dy, double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_wenork3_extend_f32(float *C, int iteration, const float *F, int rows, int cols, int pges, double dx,
                           double dy, double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);

/* ref: +SD/@SDF3/WENO5RK3ClosetPointSurfaceRedistance.m:4-157.  A is redistanced in
 * place on the zero set of F: iter1 RK3 steps, each stage preceded by iter2 extension
 * steps of A off the interface. */
int vsl_weno5_rk3_surface_redistance_f64(double *A, int iter1, int iter2, const double *F, int rows, int cols,
                                         int pges, double dx, double dy, double dz, void *workspace,
                                         size_t workspace_bytes, vsl_stream_t stream);
int vsl_weno5_rk3_surface_redistance_f32(float *A, int iter1, int iter2, const float *F, int rows, int cols,
                                         int pges, double dx, double dy, double dz, void *workspace,
                                         size_t workspace_bytes, vsl_stream_t stream);
/* ref: +SD/@SDF3/WENORK3ClosetPointSurfaceRedistance.m:4-152.  The WENORK3 form of the
 * same composition: cubic distances of A and F, the WENORK3 upwind normals of F (1e-14
 * floor), crossing values and extension step, and the reinitialization with the ENO3
 * interface scheme.  Workspace op VSL_OP_SURFACE_REDISTANCE_ENO3. */
int vsl_wenork3_surface_redistance_f64(double *A, int iter1, int iter2, const double *F, int rows, int cols,
                                       int pges, double dx, double dy, double dz, void *workspace,
                                       size_t workspace_bytes, vsl_stream_t stream);
int vsl_wenork3_surface_redistance_f32(float *A, int iter1, int iter2, const float *F, int rows, int cols,
                                       int pges, double dx, double dy, double dz, void *workspace,
                                       size_t workspace_bytes, vsl_stream_t stream);

/* ref: +SD/@SDF3/SDF3.m:73-80 (calArea, calVolume) after GPUsetCalculusToolBox.m:2-42.
 * area_volume: device pointer to 2 doubles, written with the FP64 sums
 * area = Ds^3 * sum(DiracDelta where |F| < 2Ds), volume = Ds^3 * sum(1 - Heaviside where
 * F < 2Ds), summed in a fixed order (bitwise reproducible for a given grid). */
int vsl_area_volume_f64(const double *F, double *area_volume, int rows, int cols, int pges, double dx, double dy,
                        double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_area_volume_f32(const float *F, double *area_volume, int rows, int cols, int pges, double dx, double dy,
                        double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);

/* No counterpart in the reference.  vsl_area_volume_f64 for callers that cannot allocate
 * device memory (a MEX function working on MATLAB-owned gpuArrays, a framework whose
 * allocator must not be bypassed, code that must not take cudaMalloc's implicit
 * synchronisation): no workspace argument, and the call allocates nothing.  Its scratch
 * is one static device array of VSL_NOALLOC_SCRATCH_BYTES, held by every device that loads
 * the library until the process exits.  Limit: ceil(rows/32) * ceil(cols/8) * pges <=
 * VSL_NOALLOC_SCRATCH_BYTES / 16 = 65536 (every grid up to 256^3); larger grids return
 * VSL_ERR_SCRATCH_LIMIT before anything is launched.  Every call looks up the array's
 * address on the device current at the call (nothing is cached, so the address stays right
 * after a cudaDeviceReset); the first call on a device loads the library's device code
 * there, so make that first call before any stream capture.  All calls on a device share
 * the array: calls that can overlap on the GPU race, so order them (one stream, or
 * events).  Results are bitwise those of vsl_area_volume_f64. */
#define VSL_NOALLOC_SCRATCH_BYTES 1048576
int vsl_area_volume_noalloc_f64(const double *F, double *area_volume, int rows, int cols, int pges, double dx,
                                double dy, double dz, vsl_stream_t stream);

/* WENO5 advection phi_t + v.grad(phi) = 0 (the upwind operator of
 * CUDA_Code/4_0_Calculus_ToolBox/advection_step.cu:30-56 / +SD/@GD3/GD3.m:393-398) in the
 * TVD-RK3 combination of WENO5RK3Reinitialization.m:15-39; `steps` steps of the device
 * time step *dt. */
int vsl_weno5_rk3_advection_f64(double *F, const double *vx, const double *vy, const double *vz, const double *dt,
                                int steps, int rows, int cols, int pges, double dx, double dy, double dz,
                                void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_weno5_rk3_advection_f32(float *F, const float *vx, const float *vy, const float *vz, const double *dt,
                                int steps, int rows, int cols, int pges, double dx, double dy, double dz,
                                void *workspace, size_t workspace_bytes, vsl_stream_t stream);

/* One vesicle step in the order of p00_test_singlephase_relax.m:60-196 with the normal
 * speed set to the mean curvature: calculus toolbox -> area/volume -> extend the mean
 * curvature (ext_iters WENO5 RK3 pseudo-steps) -> dt = cfl*Ds/max|Vn| over |F|<2Ds ->
 * one WENO5 RK3 advection step along Vn*N -> setDistance -> reinit_iters WENO5 RK3
 * pseudo-steps.  F and its cached distances (xpr..zpd) are updated in place.
 * info: device pointer to 4 doubles {area, volume, dt, max|Vn|} (area/volume measured
 * before the step). */
int vsl_vesicle_step_f64(double *F, double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                         int ext_iters, int reinit_iters, double cfl, double *info, int rows, int cols, int pges,
                         double dx, double dy, double dz, void *workspace, size_t workspace_bytes,
                         vsl_stream_t stream);
int vsl_vesicle_step_f32(float *F, float *xpr, float *xpl, float *ypf, float *ypb, float *zpu, float *zpd,
                         int ext_iters, int reinit_iters, double cfl, double *info, int rows, int cols, int pges,
                         double dx, double dy, double dz, void *workspace, size_t workspace_bytes,
                         vsl_stream_t stream);

/* A batch of vesicle steps, FP32 mixed form (no counterpart in the reference, which
 * advances one vesicle per MATLAB process).  Every vesicle gets the step of
 * vsl_vesicle_step_f32 (its own field, cached distances, info output and workspace of
 * vsl_workspace_bytes(VSL_OP_VESICLE_STEP, its grid, 4)); each RK stage of all the
 * vesicles runs as one launch over all their tiles, 64 vesicles at a time, and
 * the per-vesicle set-up passes stay per vesicle.  Results are bitwise those of
 * vsl_vesicle_step_f32 called per vesicle.  `vesicles` is a HOST array read during the
 * call; the pointers in it are device pointers. */
typedef struct {
    float *F;
    float *xpr, *xpl, *ypf, *ypb, *zpu, *zpd;
    double *info; /* [area, volume, dt, max |Vn|] */
    int rows, cols, pges;
    double dx, dy, dz;
    void *workspace;
    size_t workspace_bytes;
} vsl_vesicle_f32;
int vsl_vesicle_step_batch_f32(const vsl_vesicle_f32 *vesicles, int count, int ext_iters, int reinit_iters,
                               double cfl, vsl_stream_t stream);

/* A batch of WENO5RK3Reinitialization calls, FP32 mixed form (ref, per member:
 * +SD/@SDF3/WENO5RK3Reinitialization.m:3-43 with the member's cached distances, as
 * vsl_weno5_rk3_reinitialization_f32).  Each member has its own field, distances and
 * workspace of vsl_workspace_bytes(VSL_OP_REINIT_WENO5, its grid, 4); each RK stage of all
 * the members runs as one launch over all their tiles, 64 members at a time.  Results are
 * bitwise those of vsl_weno5_rk3_reinitialization_f32 called per member.  `members` is a
 * HOST array read during the call; the pointers in it are device pointers. */
typedef struct {
    float *F;
    const float *xpr, *xpl, *ypf, *ypb, *zpu, *zpd;
    int rows, cols, pges;
    double dx, dy, dz;
    void *workspace;
    size_t workspace_bytes;
} vsl_reinit_f32;
int vsl_weno5_rk3_reinitialization_batch_f32(const vsl_reinit_f32 *members, int count, int iteration,
                                             vsl_stream_t stream);

/* A batch of WENO5RK3Extend calls, FP32 mixed form (ref, per member:
 * +SD/@SDF3/WENO5RK3Extend.m:9-76 with F's cached distances, as vsl_weno5_rk3_extend_f32).
 * Each member has its own field C (extended in place), level set F, F's distances and
 * workspace of vsl_workspace_bytes(VSL_OP_EXTEND_WENO5, its grid, 4); each RK stage of all
 * the members runs as one launch over all their tiles and band blocks, 64 members at a
 * time.  Results are bitwise those of vsl_weno5_rk3_extend_f32 called per member.
 * `members` is a HOST array read during the call; the pointers in it are device
 * pointers. */
typedef struct {
    float *C;
    const float *F;
    const float *xpr, *xpl, *ypf, *ypb, *zpu, *zpd;
    int rows, cols, pges;
    double dx, dy, dz;
    void *workspace;
    size_t workspace_bytes;
} vsl_extend_f32;
int vsl_weno5_rk3_extend_batch_f32(const vsl_extend_f32 *members, int count, int iteration, vsl_stream_t stream);

/* A batch of WENO5 RK3 advections, FP32 mixed form (per member as
 * vsl_weno5_rk3_advection_f32: `steps` steps of the member's device time step *dt along its
 * velocity).  Each member has its own field F (advanced in place), velocity, time step and
 * workspace of vsl_workspace_bytes(VSL_OP_ADVECTION, its grid, 4); each RK stage of all
 * the members runs as one launch, 64 members at a time.  Results are bitwise those of
 * vsl_weno5_rk3_advection_f32 called per member.  `members` is a HOST array read during
 * the call; the pointers in it are device pointers. */
typedef struct {
    float *F;
    const float *vx, *vy, *vz;
    const double *dt;
    int rows, cols, pges;
    double dx, dy, dz;
    void *workspace;
    size_t workspace_bytes;
} vsl_advect_f32;
int vsl_weno5_rk3_advection_batch_f32(const vsl_advect_f32 *members, int count, int steps, vsl_stream_t stream);

/* A batch of closest-point surface redistances, FP32 mixed form (ref, per member:
 * +SD/@SDF3/WENO5RK3ClosetPointSurfaceRedistance.m:4-157, or for the _wenork3_ entry
 * +SD/@SDF3/WENORK3ClosetPointSurfaceRedistance.m:4-152; as
 * vsl_weno5_rk3_surface_redistance_f32 / vsl_wenork3_surface_redistance_f32).  Each member
 * has its own A (redistanced in place), F and workspace of vsl_workspace_bytes(
 * VSL_OP_SURFACE_REDISTANCE or VSL_OP_SURFACE_REDISTANCE_ENO3, its grid, 4); each RK
 * stage of the extensions and of the reinitialization of all the members runs as one
 * launch, 64 members at a time.  Results are bitwise those of the per-member calls.
 * `members` is a HOST array read during the call; the pointers in it are device
 * pointers. */
typedef struct {
    float *A;
    const float *F;
    int rows, cols, pges;
    double dx, dy, dz;
    void *workspace;
    size_t workspace_bytes;
} vsl_redistance_f32;
int vsl_weno5_rk3_surface_redistance_batch_f32(const vsl_redistance_f32 *members, int count, int iter1, int iter2,
                                               vsl_stream_t stream);
int vsl_wenork3_surface_redistance_batch_f32(const vsl_redistance_f32 *members, int count, int iter1, int iter2,
                                             vsl_stream_t stream);

/* ref: +SD/@SDF3/ENORK2Reinitialization.m:3-45.  Quadratic-ENO distances recomputed from
 * F, then `iteration` Heun RK2 pseudo-steps F1 = F - step(F), F = (F + F1 - step(F1)) / 2
 * with the mask and dt = 0.3 min(distances) of F at the start. */
int vsl_enork2_reinitialization_f64(double *F, int iteration, int rows, int cols, int pges, double dx, double dy,
                                    double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_enork2_reinitialization_f32(float *F, int iteration, int rows, int cols, int pges, double dx, double dy,
                                    double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);
/* ref: +SD/@SDF3/ENORK2Extend.m:9-81.  C extended off the zero set of F: quadratic-ENO
 * distances of F, ENO upwind normals v = sign(F) n / max(|n|, 1e-6), quadratic crossing
 * values of C, `iteration` Heun RK2 pseudo-steps. */
int vsl_enork2_extend_f64(double *C, int iteration, const double *F, int rows, int cols, int pges, double dx,
                          double dy, double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_enork2_extend_f32(float *C, int iteration, const float *F, int rows, int cols, int pges, double dx, double dy,
                          double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);
/* ref: +SD/@SDF3/ENORK2ClosetPointSurfaceRedistance.m:4-128.  A is redistanced in place
 * on the zero set of F: iter1 Heun RK2 steps with A's quadratic-ENO distances, each
 * stage preceded by iter2 ENORK2 extension steps of its input off F (normals with a
 * 1e-14 floor), and a final extension. */
int vsl_enork2_surface_redistance_f64(double *A, int iter1, int iter2, const double *F, int rows, int cols, int pges,
                                      double dx, double dy, double dz, void *workspace, size_t workspace_bytes,
                                      vsl_stream_t stream);
int vsl_enork2_surface_redistance_f32(float *A, int iter1, int iter2, const float *F, int rows, int cols, int pges,
                                      double dx, double dy, double dz, void *workspace, size_t workspace_bytes,
                                      vsl_stream_t stream);

/* ---- the single-phase relaxation step of the vesicle driver and its SD.GD3 operators -- */

/* ref: +SD/@GD3/GD3.m:344-346 (Laplacian) with the circshift neighbours of GD3.m:110-116:
 * out = (Fxx + Fyy) + Fzz, Fxx = (F(x+dx) - 2F + F(x-dx)) / Dx^2, periodic in every axis. */
int vsl_laplacian_f64(const double *field, double *out, int rows, int cols, int pges, double dx, double dy,
                      double dz, vsl_stream_t stream);
int vsl_laplacian_f32(const float *field, float *out, int rows, int cols, int pges, double dx, double dy, double dz,
                      vsl_stream_t stream);

/* ref: +SD/@GD3/GD3.m:314-318 (Gradient) of Fx, Fy, Fz (GD3.m:218-240) with the same
 * circshift neighbours: fx = (F(x+dx) - F(x-dx)) / (2 Dx), fy and fz alike, periodic in
 * every axis. */
int vsl_gradient_f64(const double *field, double *fx, double *fy, double *fz, int rows, int cols, int pges, double dx,
                     double dy, double dz, vsl_stream_t stream);
int vsl_gradient_f32(const float *field, float *fx, float *fy, float *fz, int rows, int cols, int pges, double dx,
                     double dy, double dz, vsl_stream_t stream);

/* ref: +SD/@GD3/GD3.m:434-485 (smoothGMRES, smoothFFT).  out = real(ifftn(fftn(rhs) ./ S))
 * with S = 1 + alpha * (*dt) * symbol: exact = 1 takes the symbol of the periodic discrete
 * bi-Laplacian (lambda^2, lambda = sum (2 cos(2 pi m/n) - 2) / h^2), which makes out the
 * solution of smoothGMRES's system (I + alpha Dt L^2) out = rhs; exact = 0 takes smoothFFT's
 * (kx^2 + ky^2 + kz^2)^2.  rhs and out may be the same array.  dt: device pointer.  Uses
 * cuFFT: the first call for a grid shape and precision (or vsl_workspace_bytes for
 * VSL_OP_SMOOTH / VSL_OP_RELAX_STEP) creates that shape's cuFFT plan; cuFFT allocates the
 * plan's own tables then, so make that first call before any stream capture.  The
 * transform's work area and spectrum are in the workspace. */
int vsl_smooth_bilaplacian_f64(const double *rhs, double *out, const double *dt, double alpha, int exact, int rows,
                               int cols, int pges, double dx, double dy, double dz, void *workspace,
                               size_t workspace_bytes, vsl_stream_t stream);
int vsl_smooth_bilaplacian_f32(const float *rhs, float *out, const double *dt, double alpha, int exact, int rows,
                               int cols, int pges, double dx, double dy, double dz, void *workspace,
                               size_t workspace_bytes, vsl_stream_t stream);

/* ref: p00_test_singlephase_relax.m:60-196 (one pass of the time loop, without plotting).
 * Calculus toolbox of F -> area, volume -> H = WENORK3Extend(MeanCurvature, ext_iters) ->
 * NSB = kappa (Laplacian(H) + 0.5 H (H^2 - 4K) + 2 c0 K - 0.5 c0^2 H) ->
 * NSB = ENORK2Extend(NSB, ext_iters) -> Dt = cfl Ds / max|NSB| over |F| < 2Ds ->
 * [tension; pressure] = [c11 c12; c12 A0] \ [s1; s2] from the surface integrals ->
 * v = (tension H - NSB + pressure) |grad F| -> (I + alpha Dt L^2)^-1 v (exact spectral
 * solve of smoothGMRES's system) -> ENORK2Extend(v, ext_iters) -> F = F - Dt v ->
 * setDistance (F's cached distances xpr..zpd are rewritten) -> energy -> reinit_iters
 * WENO5 RK3 reinitialization pseudo-steps (0: none; the driver reinitializes every
 * ReinitializationRate steps).  A0, V0: the initial area and volume; c0 = spon_c.
 * info: device pointer to 11 doubles {area, volume (at the start), Dt, max|NSB|, c11 =
 * int H^2, c12 = int H, int H NSB, int NSB, tension, pressure, energy int (H - c0)^2}. */
int vsl_relax_step_f64(double *F, double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                       double A0, double V0, double kappa, double spon_c, double cfl, double alpha, int ext_iters,
                       int reinit_iters, double *info, int rows, int cols, int pges, double dx, double dy, double dz,
                       void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_relax_step_f32(float *F, float *xpr, float *xpl, float *ypf, float *ypb, float *zpu, float *zpd, double A0,
                       double V0, double kappa, double spon_c, double cfl, double alpha, int ext_iters,
                       int reinit_iters, double *info, int rows, int cols, int pges, double dx, double dy, double dz,
                       void *workspace, size_t workspace_bytes, vsl_stream_t stream);

/* ---- the auxiliary level set of multiphase vesicles ----------------------------------
 *
 * A second level set A marks the domains on the vesicle surface F = 0; its zero set on the
 * surface is the domain boundary (a curve). */

/* ref: CUDA_Code/4_0_Calculus_ToolBox/auxi_set_calculus_toolbox.cu:10-11 (drop-in, FP64):
 * A's central differences, the curve tangent t = (grad F x grad A) / |.|, the conormal
 * n = t x N, geodesic and normal curvature, geodesic torsion, BPerpendicular, and A's
 * Heaviside/Dirac functions from AHPrimal = max(A, 0); F's toolbox fields are inputs.
 * Every output is written at every node. */
int vsl_auxi_set_calculus_toolbox(
    double *Ax, double *Ay, double *Az, double *AGradMag, double *Cx, double *Cy, double *Cz, double *NormCrossAF,
    double *tx, double *ty, double *tz, double *nx, double *ny, double *nz, double *Axx, double *Ayy, double *Azz,
    double *Axy, double *Ayz, double *Azx, double *ALaplacian, double *GeodesicCurvature, double *NormalCurvature,
    double *GeodesicTorsion, double *BPerpendicular, double *AHeaviside, double *ADiracDelta, const double *lsf,
    const double *AHPrimal, const double *Fx, const double *Fy, const double *Fz, const double *FGradMag,
    const double *Nx, const double *Ny, const double *Nz, const double *Fxx, const double *Fyy, const double *Fzz,
    const double *Fxy, const double *Fyz, const double *Fzx, int rows, int cols, int pges, double dx, double dy,
    double dz, double ds, int num_ele, vsl_stream_t stream);

/* ref: +SD/@SDF3/GPUAsetCalculusToolBox.m:2-63.  The auxiliary toolbox of A on F, reading
 * only A and F (F's gradient, Hessian, normal and Heaviside function are recomputed with
 * the calculus toolbox's own expressions).  out: a host array of 29 device pointers, the
 * 27 fields of vsl_auxi_set_calculus_toolbox in its order, then AFDiracDelta = (C . (grad
 * H_F x grad H_A)) / |C|^2 and ADiracDeltaDn = (Laplacian(AHeaviside) - ADiracDelta
 * Laplacian(A)) / |grad A| (GD3's periodic operators); a null entry is not written.
 * Ds = (dx + dy + dz) / 3.  Workspace op VSL_OP_AUX_TOOLBOX. */
int vsl_a_set_calculus_toolbox_f64(const double *A, const double *F, double *const *out, int rows, int cols,
                                   int pges, double dx, double dy, double dz, void *workspace,
                                   size_t workspace_bytes, vsl_stream_t stream);
int vsl_a_set_calculus_toolbox_f32(const float *A, const float *F, float *const *out, int rows, int cols,
                                   int pges, double dx, double dy, double dz, void *workspace,
                                   size_t workspace_bytes, vsl_stream_t stream);

/* ref: +SD/@SDF3/SDF3.m:82-85 (surfaceIntegral), 212-219 (calLength, LineIntegral),
 * 220-227 (AcalArea, AsurfaceIntegral).  *result (device) = Ds^3 times the FP64 sum over
 * the nodes with |F| < 2Ds (and |A| < 2Ds where A is not null) of ((f0 f1) f2)
 * (1 - one_minus), a null factor left out (a null f0 counts as 1):
 *   surfaceIntegral(f)  = (F, null, f, DiracDelta, FGradMag, null)
 *   calLength           = (F, A, AFDiracDelta, NormCrossAF, null, null)
 *   LineIntegral(f)     = (F, A, f, AFDiracDelta, NormCrossAF, null)
 *   AcalArea            = (F, null, DiracDelta, null, null, AHeaviside)
 *   AsurfaceIntegral(f) = (F, null, f, DiracDelta, FGradMag, AHeaviside)
 * Workspace op VSL_OP_MASKED_INTEGRAL. */
int vsl_masked_integral_f64(const double *F, const double *A, const double *f0, const double *f1,
                            const double *f2, const double *one_minus, double *result, int rows, int cols, int pges,
                            double dx, double dy, double dz, void *workspace, size_t workspace_bytes,
                            vsl_stream_t stream);
int vsl_masked_integral_f32(const float *F, const float *A, const float *f0, const float *f1, const float *f2,
                            const float *one_minus, double *result, int rows, int cols, int pges, double dx,
                            double dy, double dz, void *workspace, size_t workspace_bytes, vsl_stream_t stream);

/* ---- adjoints (no counterpart in the reference, which has no derivatives) -------------
 *
 * Reverse-mode sweeps of the forward operations above, for gradients of a loss L of a
 * transported and reinitialized field.  Each recomputes what it needs of its forward
 * pass from the forward input with the same kernels, and differentiates every update as
 * the forward evaluated it (WENO weights with their epsilon, upwind and Godunov switches,
 * the interface insertion, the min over the six distances).
 *
 * One WENO5 TVD-RK3 advection step F -> F' (vsl_weno5_rk3_advection_* with steps = 1)
 * with the fixed time step *dt.  lam: on entry dL/dF', on return dL/dF.
 * gvx, gvy, gvz: dL/dv of this step is ADDED (accumulate over steps; zero them first). */
int vsl_weno5_rk3_advection_adjoint_f64(const double *F, const double *vx, const double *vy, const double *vz,
                                        const double *dt, double *lam, double *gvx, double *gvy, double *gvz,
                                        int rows, int cols, int pges, double dx, double dy, double dz,
                                        void *workspace, size_t workspace_bytes, vsl_stream_t stream);
int vsl_weno5_rk3_advection_adjoint_f32(const float *F, const float *vx, const float *vy, const float *vz,
                                        const double *dt, float *lam, float *gvx, float *gvy, float *gvz, int rows,
                                        int cols, int pges, double dx, double dy, double dz, void *workspace,
                                        size_t workspace_bytes, vsl_stream_t stream);

/* The reinitialization F0 -> F' of setDistance (degree-5 roots) followed by
 * vsl_weno5_rk3_reinitialization_* with `iteration` pseudo-steps.  lam: on entry dL/dF',
 * on return dL/dF0, including the path through the interface distances (the
 * implicit-function derivative of each root).  tape: device buffer of
 * iteration * rows*cols*pges elements, overwritten with the pseudo-step inputs. */
int vsl_weno5_rk3_reinitialization_adjoint_f64(const double *F0, int iteration, double *lam, double *tape, int rows,
                                               int cols, int pges, double dx, double dy, double dz, void *workspace,
                                               size_t workspace_bytes, vsl_stream_t stream);
int vsl_weno5_rk3_reinitialization_adjoint_f32(const float *F0, int iteration, float *lam, float *tape, int rows,
                                               int cols, int pges, double dx, double dy, double dz, void *workspace,
                                               size_t workspace_bytes, vsl_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif
