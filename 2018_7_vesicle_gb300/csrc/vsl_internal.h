// vsl_internal.h -- shared declarations between the translation units of the library.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/vsl_gb300.h"
#include "vsl_device.cuh"

// NVTX ranges around the C-ABI operations (named after the operation) for timeline
// profilers; compiled in only with -DVSL_NVTX, a no-op statement otherwise
#if defined(VSL_NVTX) && __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
namespace vsl {
struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};
}  // namespace vsl
#define VSL_RANGE(name) ::vsl::TraceRange vsl_trace_range_(name)
#else
#define VSL_RANGE(name) (void)0
#endif

namespace vsl {

// thread block used by the node-parallel kernels: 32 rows x 8 columns of one page
constexpr int BX = 32;
constexpr int BY = 8;

inline dim3 node_grid(const Grid &g) { return dim3((g.rows + BX - 1) / BX, (g.cols + BY - 1) / BY, g.pges); }

// Validation shared by every entry point (status codes of vsl_gb300.h).
inline int check_grid(int rows, int cols, int pges, double dx, double dy, double dz)
{
    if (rows <= 0 || cols <= 0 || pges <= 0) return VSL_ERR_SHAPE;
    if ((long long)rows * cols * pges > (long long)VSL_MAX_NODES) return VSL_ERR_SHAPE;
    if (pges > 65535) return VSL_ERR_SHAPE;
    if (!(dx > 0) || !(dy > 0) || !(dz > 0)) return VSL_ERR_VALUE;
    return VSL_OK;
}

inline int launch_status(cudaError_t e) { return e == cudaSuccess ? VSL_OK : VSL_ERR_CUDA; }

template <typename T> struct Ptr6 {
    T *p[6];
};
template <typename T> struct Ptr3 {
    T *p[3];
};

// compact lists built on the device: node indices and their count (zeroed by the launcher)
struct NodeList {
    unsigned *idx;
    unsigned *count;
};
// one list of crossed edges per axis (the node at the edge's lower end), counts [3]
struct EdgeLists {
    unsigned *idx[3];
    unsigned *count;
};

// ---- fused kernels (vsl_fused.cuh), T in {float, double} -------------------------------
// setDistance: defaults plus a list of crossed edges, then one root per listed edge
template <typename T>
cudaError_t launch_set_distance(const T *phi, Ptr6<T> dist, const Grid &g, bool quintic, EdgeLists e,
                                cudaStream_t s);
// classification bytes; with list.idx non-null also the list of nodes with a distance flag
template <typename T>
cudaError_t launch_classify(const T *phi0, Ptr6<const T> dist, uint8_t *flags, NodeList list, const Grid &g,
                            cudaStream_t s);
template <typename T>
cudaError_t launch_reinit_stage(const T *phi_s, const T *phi_n, T *out, const uint8_t *flags, Ptr6<const T> dist,
                                const Grid &g, int stage, bool eno3, bool fast, cudaStream_t s);
// flags: the classification bytes of phi with these distances (launch_classify); flagged:
// its list of flagged nodes (the FP32 form then runs the uniform nodes and the list apart)
template <typename T>
cudaError_t launch_extension_velocity(const T *phi, const uint8_t *flags, Ptr6<const T> dist, Ptr3<T> v, const Grid &g,
                                      bool eno3, double floor, NodeList flagged, cudaStream_t s);
// crossing values at the listed (flagged) nodes only; other entries of cp are not written
template <typename T>
cudaError_t launch_crossing(const T *c, Ptr6<const T> dist, Ptr6<T> cp, NodeList list, const Grid &g, bool cubic,
                            cudaStream_t s);
template <typename T>
cudaError_t launch_extend_stage(const T *c_s, const T *c_n, T *out, const uint8_t *flags, Ptr6<const T> dist,
                                Ptr6<const T> cp, Ptr3<const T> v, const Grid &g, int stage, bool eno3, bool fast,
                                cudaStream_t s);
template <typename T>
cudaError_t launch_advect_stage(const T *phi_s, const T *phi_n, T *out, Ptr3<const T> v, const T *speed,
                                const double *dt, const Grid &g, int stage, bool fast, cudaStream_t s);

// Reinitialization residual (no counterpart in the reference, whose loops run a fixed
// count): the FP64 maximum over the band |phi| < band of | |grad phi|_G - 1 |, the Godunov
// norm the stage takes, at the non-fixed nodes.  The last block to finish records it and
// decides whether a residual-driven loop goes on (see ResidualState).
struct ResidualState {
    unsigned long long *max_bits;  // running maximum, the bits of a non-negative double (zero between uses)
    unsigned *ticket;              // blocks finished (zero between uses)
    int *status;                   // [pseudo-steps done, 1 if the residual is <= tol]
    double *history;               // residual after each pseudo-step, [0] on entry (may be null)
    unsigned *zero_counter;        // a band counter the next pseudo-step needs zeroed (may be null)
    double tol;
    int cap;                       // most pseudo-steps
    int advance;                   // 1: one more pseudo-step was taken before this evaluation
    int has_handle;                // inside a residual-driven loop (a conditional graph node)
    cudaGraphConditionalHandle handle;  // the loop's condition, set to (residual > tol && steps < cap)
};
template <typename T>
cudaError_t launch_reinit_residual(const T *phi, const uint8_t *flags, Ptr6<const T> dist, const Grid &g, double band,
                                   const ResidualState &st, cudaStream_t s);
// 1 thread: the loop condition of a residual-driven loop set to 0 (the first node of each
// iteration, so that only a completed residual evaluation can continue the loop)
cudaError_t launch_condition_reset(cudaGraphConditionalHandle handle, cudaStream_t s);

// ENORK2 (second-order ENO, Heun RK2 stages 0 and 1): quadratic-ENO distances, the
// reinitialization and extension stages, the extension velocity and crossing values
template <typename T>
cudaError_t launch_set_distance_eno2(const T *phi, Ptr6<T> dist, const Grid &g, EdgeLists e, cudaStream_t s);
template <typename T>
cudaError_t launch_enork2_reinit_stage(const T *phi_s, const T *phi_n, T *out, const uint8_t *flags,
                                       Ptr6<const T> dist, const Grid &g, int stage, cudaStream_t s);
template <typename T>
cudaError_t launch_enork2_velocity(const T *phi, Ptr6<const T> dist, Ptr3<T> v, const Grid &g, double floor,
                                   cudaStream_t s);
template <typename T>
cudaError_t launch_enork2_crossing(const T *c, Ptr6<const T> dist, Ptr6<T> cp, NodeList list, const Grid &g,
                                   cudaStream_t s);
template <typename T>
cudaError_t launch_enork2_extend_stage(const T *c_s, const T *c_n, T *out, const uint8_t *flags, Ptr6<const T> dist,
                                       Ptr6<const T> cp, Ptr3<const T> v, const Grid &g, int stage, cudaStream_t s);

// ---- the relaxation step (vsl_relax.cuh, vsl_spectral.cu), T in {float, double} ------
template <typename T> cudaError_t launch_laplacian(const T *f, T *out, const Grid &g, cudaStream_t s);
template <typename T>
cudaError_t launch_gradient(const T *f, T *fx, T *fy, T *fz, const Grid &g, cudaStream_t s);
template <typename T>
cudaError_t launch_bending_speed(const T *H, const T *K, T *out, const Grid &g, double kappa, double c0,
                                 cudaStream_t s);
// per-block partials of the surface integrals over |F| < band: 4 (H^2, H, H NSB, NSB) or,
// with energy, 1 ((H - c0)^2)
template <typename T>
cudaError_t launch_relax_moments(const T *F, const T *H, const T *nsb, const T *delta, const T *gmag, double band,
                                 double c0, bool energy, const Grid &g, double *partials, int *nblocks, cudaStream_t s);
cudaError_t launch_tension_pressure(const double *moments, const double *area_volume, const double *dt, double A0,
                                    double V0, double *tp, cudaStream_t s);
template <typename T>
cudaError_t launch_normal_speed(const T *H, const T *nsb, const T *gmag, const double *tp, T *out, const Grid &g,
                                cudaStream_t s);
template <typename T> cudaError_t launch_euler(T *F, const T *v, const double *dt, const Grid &g, cudaStream_t s);
// cuFFT work bytes of a shape (creates the shape's plan on first use; 0 on failure)
template <typename T> size_t spectral_work_bytes(const Grid &g);
// out = real(ifftn(fftn(rhs) ./ (1 + alpha dt symbol))); spectrum: num complex elements
template <typename T>
int launch_smooth_bilaplacian(const T *rhs, T *out, const double *dt, double alpha, bool exact, const Grid &g,
                              void *spectrum, void *work, size_t work_bytes, cudaStream_t s);

// ---- tiled FP32 stage kernels (vsl_tiled.cuh, built into vsl_fused_f32.cu) ----------
// compact queue of the nodes that need the interface-aware stencil, two counters used
// alternately by consecutive stages (zeroed at the start of an operation)
struct BandQueue {
    unsigned *queue;
    unsigned *counter;
};
// The mixed form's FP64 interface data of an extension stage: the crossing values and an
// FP64 copy ("shadow") of the flagged nodes' values of the stage input, the step-start
// field and the stage output.  A one-sided divided difference across a short gap g between
// a node and a crossing, (C_node - C_cross) / g, amplifies the FP32 rounding of C_node and
// C_cross by h / g (a gap of 2e-4 h turns an FP32 ulp into a 5e-3 relative error of the
// derivative), so those values stay FP64 where the band kernel forms such differences.
struct BandShadow {
    const double *s_in;
    const double *s_n;
    double *s_out;
    Ptr6<const double> cp;
};
struct TiledStage {
    const float *phi_s;
    const float *phi_n;
    float *out;
    const uint8_t *flags;
    Ptr6<const float> d;
    BandShadow shadow;  // extension kinds only
    Ptr3<const float> v;
    const float *speed;
    const double *dt;
    BandQueue band;   // reinitialization: nodes queued by the stage kernel
    NodeList flagged; // extension: the static list of nodes with a distance flag
    int stage;        // 0, 1, 2 within the RK3 step
    int seq;          // running stage count since the counters were zeroed
};
// kind: 0 reinitialization, 1 extension, 2 advection
cudaError_t launch_tiled_stage(int kind, bool eno3, const TiledStage &st, const Grid &g, cudaStream_t s);
// plane loads of the 2.5D-tiled stage kernels: 1 = TMA for the inner tiles, 0 = registers
int set_plane_loads(int mode);
int get_plane_loads();
cudaError_t tma_timeouts(unsigned *count);
// the mixed form's extension velocity of the nodes without a distance flag, on 2.5D tiles
cudaError_t launch_velocity_tiled(const float *phi, const uint8_t *flags, Ptr3<float> v, const Grid &g, float floor,
                                  cudaStream_t s);
// the same stage (same kind and RK stage) of `count` <= TILED_BATCH_MAX grids as one
// launch over all their tiles, and one launch for all their band nodes
constexpr int TILED_BATCH_MAX = 64;
cudaError_t launch_tiled_batch(int kind, bool eno3, const TiledStage *st, const Grid *grids, int count, cudaStream_t s);
// the mixed form's extension set-up at the listed (flagged) nodes: FP64 crossing values on
// the promoted FP32 field (degree-5 / cubic product form, or the ENORK2 quadratic), and the
// shadow of the field's values
cudaError_t launch_crossing_mixed(const float *c, Ptr6<const float> dist, Ptr6<double> cp, NodeList list,
                                  const Grid &g, bool cubic, cudaStream_t s);
cudaError_t launch_enork2_crossing_mixed(const float *c, Ptr6<const float> dist, Ptr6<double> cp, NodeList list,
                                         const Grid &g, cudaStream_t s);
cudaError_t launch_shadow_init(const float *c, double *shadow, NodeList list, cudaStream_t s);
// pages per block of the tiled kernels for a grid shape and kind (the tuning table, or the
// default); set_tile_pages(..., 0) restores the default
int tile_pages(const Grid &g, int kind);
int set_tile_pages(int rows, int cols, int pges, int kind, int pages);

// ---- toolbox and reductions (vsl_toolbox.cu) ------------------------------------------
// Fields of the calculus toolbox a caller may ask for (null pointers are skipped).
template <typename T> struct ToolboxOut {
    T *f[18];
};
template <typename T>
cudaError_t launch_toolbox(const T *phi, ToolboxOut<T> out, const Grid &g, double ds, double *partials,
                           int *nblocks, cudaStream_t s);
cudaError_t launch_sum_partials(const double *partials, int nblocks, int ncomp, double scale, double *result,
                                cudaStream_t s);
template <typename T>
cudaError_t launch_band_maxabs(const T *f, const T *phi, double band, const Grid &g, double *partials,
                               int *nblocks, cudaStream_t s);
cudaError_t launch_time_step(const double *partials, int nblocks, double cfl_ds, double *dt, double *vmax,
                             cudaStream_t s);
int toolbox_partial_blocks(const Grid &g);

// ---- auxiliary level set toolbox and masked integrals (vsl_auxi.cuh) -------------------
// The 27 fields of auxi_set_calculus_toolbox in its argument order, then AFDiracDelta and
// ADiracDeltaDn (null pointers are skipped).
constexpr int AUX_OUT_FIELDS = 29;
template <typename T> struct AuxOut {
    T *f[AUX_OUT_FIELDS];
};
// F's toolbox inputs of the reference kernel: Fx Fy Fz FGradMag Nx Ny Nz Fxx Fyy Fzz Fxy Fyz Fzx
template <typename T> struct AuxFIn {
    const T *f[13];
};
// per-node values pass 2 of the fused form reads (outputs or workspace)
template <typename T> struct AuxKeep {
    T *cx, *cy, *cz, *ncr, *agm, *adelta, *aheav, *fheav;
};
template <typename T> struct AuxKeepC {
    const T *cx, *cy, *cz, *ncr, *agm, *adelta, *aheav, *fheav;
};
template <typename T>
cudaError_t launch_aux_toolbox(const T *A, const T *F, AuxOut<T> o, AuxKeep<T> keep, const Grid &g, double ds,
                               cudaStream_t s);
cudaError_t launch_auxi_dropin(AuxOut<double> o, const double *lsf, const double *ahp, AuxFIn<double> fin,
                               const Grid &g, double ds, cudaStream_t s);
// per-block FP64 partials of the masked product sum (see k_masked_sum)
template <typename T>
cudaError_t launch_masked_sum(const T *F, const T *A, const T *f0, const T *f1, const T *f2, const T *om,
                              const Grid &g, double ds, double *partials, int *nblocks, cudaStream_t s);

// ---- adjoint kernels (vsl_adjoint.cu), T in {float, double} ------------------------
// W: 21 slot fields of g.num values each (slot ax*7 + o: line offset o - 3 along ax)
template <typename T>
cudaError_t launch_adj_advect_jac(const T *ps, Ptr3<const T> v, const double *dt, const T *lam, double coef, T *W,
                                  Ptr3<T> gv, const Grid &g, cudaStream_t s);
// band: scratch list (g.num entries + a counter) of the nodes next to a sign change
template <typename T>
cudaError_t launch_adj_reinit_jac(const T *ps, const uint8_t *flags, Ptr6<const T> d, const T *lam, double coef, T *W,
                                  Ptr6<T> mu, NodeList band, const Grid &g, cudaStream_t s);
template <typename T>
cudaError_t launch_adj_gather(const T *W, const T *lam, double alpha, const T *acc, T *out, const Grid &g,
                              cudaStream_t s);
template <typename T>
cudaError_t launch_adj_axpy(T *acc, const T *lam, double a, bool init, const Grid &g, cudaStream_t s);
template <typename T>
cudaError_t launch_adj_dist_edges(const T *f, EdgeLists e, Ptr6<const T> mu, T *W, const Grid &g, cudaStream_t s);
constexpr int ADJ_SLOTS = 21;

}  // namespace vsl
