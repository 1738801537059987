// vsl_plain.cu -- FP64 drop-in kernels with the reference kernels' argument order and
// in/out semantics, one thread per node.  Each kernel restates one reference kernel
// (cited per kernel) with the same arithmetic; the neighbour gathers use 64-bit clamped
// indices and read-only loads.
#include "vsl_internal.h"

namespace vsl {
namespace {

struct Fields6 {
    double *p[6];
};
struct CFields6 {
    const double *p[6];
};

__device__ __forceinline__ bool node_of_thread(const Grid &g, int &i, int &j, int &k)
{
    i = blockIdx.x * BX + threadIdx.x;
    j = blockIdx.y * BY + threadIdx.y;
    k = blockIdx.z;
    return i < g.rows && j < g.cols;
}

// boundary_location / boundary_correction in gather form: each node writes its own
// forward distance when the interface crosses its +1 edge and its own backward distance
// when it crosses its -1 edge (h minus the -1 neighbour's forward distance, recomputed
// from the same inputs).  The set of entries written, and their values, are those of
// the reference's scatter form (boundary_location.cu:84-132), without two threads
// touching one element.
template <bool QUINTIC>
__global__ void __launch_bounds__(BX *BY) k_boundary_location(Fields6 d, const double *__restrict__ f, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    const double f0 = __ldg(f + c);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        AxisLine L = axis_line(g, i, j, k, ax);
        const double h = axis_h(g, ax);
        const double fn = __ldg(f + L.base + (long long)clampi(L.c + 1, L.n) * L.stride);
        if (f0 * fn < 0) d.p[2 * ax][c] = fore_distance<QUINTIC>(f, L, h);
        if (L.c > 0) {
            const double fp = __ldg(f + L.base + (long long)(L.c - 1) * L.stride);
            if (fp * f0 < 0) {
                AxisLine Lp = L;
                Lp.c = L.c - 1;
                d.p[2 * ax + 1][c] = h - fore_distance<QUINTIC>(f, Lp, h);
            }
        }
    }
}

// re_step (re_step.cu:283-393; ENO3: weno_rk3_reinitialization.cu:295-406).
template <bool ENO3>
__global__ void __launch_bounds__(BX *BY) k_re_step(double *__restrict__ step, const double *__restrict__ lsf,
                                                      const bool *__restrict__ mask, const double *__restrict__ deltat,
                                                      CFields6 d, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    const double tiny = 1e-6 * g.dx;
    double r[3], l[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        r[ax] = __ldg(d.p[2 * ax] + c);
        l[ax] = __ldg(d.p[2 * ax + 1] + c);
    }
    if (r[0] < tiny || l[0] < tiny || r[1] < tiny || l[1] < tiny || r[2] < tiny || l[2] < tiny) {
        step[c] = 0;
        return;
    }
    double df[3], db[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7];
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        const double h = axis_h(g, ax);
        if (p[2] * p[3] < 0 || p[3] * p[4] < 0)
            interface_pair(p, r[ax], l[ax], h, 0.0, 0.0, ENO3, df[ax], db[ax]);
        else
            weno5_pair_plain(p, h, df[ax], db[ax]);
    }
    const bool neg = mask[c];
    const double gn = godunov_norm(neg, df[0], db[0], df[1], db[1], df[2], db[2]);
    step[c] = (gn - 1) * __ldg(deltat + c) * (neg ? -1. : 1.);
}

// upwind_normal (upwind_normal.cu:4-104; wenork3_extend.cu:192-292).
template <bool ENO3>
__global__ void __launch_bounds__(BX *BY) k_upwind_normal(Fields6 n, const double *__restrict__ lsf, CFields6 d, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7], df, db;
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        const double h = axis_h(g, ax);
        const double r1 = __ldg(d.p[2 * ax] + c), l1 = __ldg(d.p[2 * ax + 1] + c);
        if (r1 < h || l1 < h)
            interface_pair(p, r1, l1, h, 0.0, 0.0, ENO3, df, db);
        else
            weno5_pair_plain(p, h, df, db);
        n.p[ax][c] = (fabs(p[4]) < fabs(p[2])) ? df : db;
    }
}

// boundary_interpolant (boundary_interpolant.cu:102-141) / boundary_interpolate
// (wenork3_extend.cu:331-365): the field's value at each crossing, 0 elsewhere.
template <bool CUBIC>
__global__ void __launch_bounds__(BX *BY) k_crossing_plain(Fields6 cp, CFields6 d, const double *__restrict__ lsf, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7], cf, cb;
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        const double h = axis_h(g, ax);
        const double r1 = __ldg(d.p[2 * ax] + c), l1 = __ldg(d.p[2 * ax + 1] + c);
        if (CUBIC)
            crossing_cubic(p, r1, l1, h, cf, cb);
        else
            crossing_quintic(p, r1, l1, h, cf, cb);
        cp.p[2 * ax][c] = cf;
        cp.p[2 * ax + 1][c] = cb;
    }
}

// extend_step (extend_step.cu:10-125; wenork3_extend.cu:372-487).
template <bool ENO3>
__global__ void __launch_bounds__(BX *BY) k_extend_step(double *__restrict__ step, const double *__restrict__ deltat,
                                                          const double *__restrict__ lsf, CFields6 v3, CFields6 d,
                                                          CFields6 cp, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    const double tiny = 1e-6 * g.dx;
    double r[3], l[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        r[ax] = __ldg(d.p[2 * ax] + c);
        l[ax] = __ldg(d.p[2 * ax + 1] + c);
    }
    if (r[0] < tiny || l[0] < tiny || r[1] < tiny || l[1] < tiny || r[2] < tiny || l[2] < tiny) {
        step[c] = 0;
        return;
    }
    double df[3], db[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7];
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        const double h = axis_h(g, ax);
        if (r[ax] < h || l[ax] < h)
            interface_pair(p, r[ax], l[ax], h, __ldg(cp.p[2 * ax] + c), __ldg(cp.p[2 * ax + 1] + c), ENO3, df[ax],
                           db[ax]);
        else
            weno5_pair_plain(p, h, df[ax], db[ax]);
    }
    step[c] = upwind_dot(__ldg(v3.p[0] + c), __ldg(v3.p[1] + c), __ldg(v3.p[2] + c), df[0], db[0], df[1], db[1],
                         df[2], db[2]) *
              __ldg(deltat + c);
}

// advection_step (advection_step.cu:30-56) and weno_derivative
// (nonoscillating_interpolant.cu:59-122).
__global__ void __launch_bounds__(BX *BY) k_advection_step(double *__restrict__ out, CFields6 v3,
                                                             const double *__restrict__ lsf, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    double df[3], db[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7];
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        weno5_pair_plain(p, axis_h(g, ax), df[ax], db[ax]);
    }
    out[c] = upwind_dot(__ldg(v3.p[0] + c), __ldg(v3.p[1] + c), __ldg(v3.p[2] + c), df[0], db[0], df[1], db[1],
                        df[2], db[2]);
}

__global__ void __launch_bounds__(BX *BY) k_weno_derivative(Fields6 out, const double *__restrict__ lsf, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7], df, db;
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        weno5_pair_plain(p, axis_h(g, ax), df, db);
        out.p[2 * ax][c] = db;
        out.p[2 * ax + 1][c] = df;
    }
}

// set_calculus_toolbox (set_calculus_toolbox.cu:9-107).
struct Fields18 {
    double *p[18];
};

__global__ void __launch_bounds__(BX *BY) k_set_calculus_toolbox(Fields18 o, const double *__restrict__ f,
                                                                   const double *__restrict__ hp, Grid g, double ds)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    const long long xp = clamped_index(g, i, j + 1, k), xm = clamped_index(g, i, j - 1, k);
    const long long yp = clamped_index(g, i + 1, j, k), ym = clamped_index(g, i - 1, j, k);
    const long long zp = clamped_index(g, i, j, k + 1), zm = clamped_index(g, i, j, k - 1);
    const double dx = g.dx, dy = g.dy, dz = g.dz;
    const double fc = __ldg(f + c);
    double fx = (__ldg(f + xp) - __ldg(f + xm)) / (2 * dx);
    double fy = (__ldg(f + yp) - __ldg(f + ym)) / (2 * dy);
    double fz = (__ldg(f + zp) - __ldg(f + zm)) / (2 * dz);
    double gm = vmax(sqrt(fx * fx + fy * fy + fz * fz), 1e-14);
    double fxx = (__ldg(f + xp) - 2 * fc + __ldg(f + xm)) / (dx * dx);
    double fyy = (__ldg(f + yp) - 2 * fc + __ldg(f + ym)) / (dy * dy);
    double fzz = (__ldg(f + zp) - 2 * fc + __ldg(f + zm)) / (dz * dz);
    double fxy = (__ldg(f + clamped_index(g, i + 1, j + 1, k)) + __ldg(f + clamped_index(g, i - 1, j - 1, k)) -
                  __ldg(f + clamped_index(g, i + 1, j - 1, k)) - __ldg(f + clamped_index(g, i - 1, j + 1, k))) /
                 (4 * ds * ds);
    double fyz = (__ldg(f + clamped_index(g, i + 1, j, k + 1)) + __ldg(f + clamped_index(g, i - 1, j, k - 1)) -
                  __ldg(f + clamped_index(g, i + 1, j, k - 1)) - __ldg(f + clamped_index(g, i - 1, j, k + 1))) /
                 (4 * ds * ds);
    double fzx = (__ldg(f + clamped_index(g, i, j + 1, k + 1)) + __ldg(f + clamped_index(g, i, j - 1, k - 1)) -
                  __ldg(f + clamped_index(g, i, j + 1, k - 1)) - __ldg(f + clamped_index(g, i, j - 1, k + 1))) /
                 (4 * ds * ds);
    double lap = fxx + fyy + fzz;
    double r1 = fxx * fx + fxy * fy + fzx * fz;
    double r2 = fxy * fx + fyy * fy + fyz * fz;
    double r3 = fzx * fx + fyz * fy + fzz * fz;
    double mean = -lap / gm + (fx * r1 + fy * r2 + fz * r3) / pow_cr<3>(gm);
    r1 = (fyy * fzz - fyz * fyz) * fx + (fzx * fyz - fxy * fzz) * fy + (fxy * fyz - fzx * fyy) * fz;
    r2 = (fyz * fzx - fxy * fzz) * fx + (fxx * fzz - fzx * fzx) * fy + (fzx * fxy - fxx * fyz) * fz;
    r3 = (fxy * fyz - fyy * fzx) * fx + (fzx * fxy - fxx * fyz) * fy + (fxx * fyy - fxy * fxy) * fz;
    double gm2 = gm * gm;
    const double gm4 = pow_cr<4>(gm);
    double gauss = (fx * r1 + fy * r2 + fz * r3) / gm4;
    double px = (__ldg(hp + xp) - __ldg(hp + xm)) / (2 * dx);
    double py = (__ldg(hp + yp) - __ldg(hp + ym)) / (2 * dy);
    double pz = (__ldg(hp + zp) - __ldg(hp + zm)) / (2 * dz);
    double dot = px * fx + py * fy + pz * fz;
    const double hc = __ldg(hp + c);
    double pxx = (__ldg(hp + xp) - 2 * hc + __ldg(hp + xm)) / (dx * dx);
    double pyy = (__ldg(hp + yp) - 2 * hc + __ldg(hp + ym)) / (dy * dy);
    double pzz = (__ldg(hp + zp) - 2 * hc + __ldg(hp + zm)) / (dz * dz);
    double plap = pxx + pyy + pzz;
    const double vals[18] = {fx,  fy,  fz,  gm,  fx / gm, fy / gm, fz / gm, fxx, fyy, fzz, fxy, fyz, fzx, lap, mean,
                             gauss, dot / gm2, plap / gm2 - dot * lap / gm4};
#pragma unroll
    for (int q = 0; q < 18; ++q) o.p[q][c] = vals[q];
}

// ---- ENORK2 (1_0_ENORK2_Reinitialization/boundary_correction.cu,
//      2_0_ENORK2_Extend/enork2_extend.cu) ---------------------------------------------

// boundary_correction (ENORK2, boundary_correction.cu:104-146) in the gather form of
// k_boundary_location: quadratic-ENO distances only.
__global__ void __launch_bounds__(BX *BY) k_enork2_boundary_correction(Fields6 d, const double *__restrict__ f, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    const double f0 = __ldg(f + c);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        AxisLine L = axis_line(g, i, j, k, ax);
        const double h = axis_h(g, ax);
        const double fn = __ldg(f + L.base + (long long)clampi(L.c + 1, L.n) * L.stride);
        if (f0 * fn < 0) d.p[2 * ax][c] = eno2_fore_distance(f, L, h);
        if (L.c > 0) {
            const double fp = __ldg(f + L.base + (long long)(L.c - 1) * L.stride);
            if (fp * f0 < 0) {
                AxisLine Lp = L;
                Lp.c = L.c - 1;
                d.p[2 * ax + 1][c] = h - eno2_fore_distance(f, Lp, h);
            }
        }
    }
}

// re_step (ENORK2, boundary_correction.cu:148-200): no fixed-node test.
__global__ void __launch_bounds__(BX *BY) k_enork2_re_step(double *__restrict__ step, const double *__restrict__ lsf,
                                                             const bool *__restrict__ mask,
                                                             const double *__restrict__ deltat, CFields6 d, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    double df[3], db[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7];
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        eno2_pair(p, __ldg(d.p[2 * ax] + c), __ldg(d.p[2 * ax + 1] + c), axis_h(g, ax), 0.0, 0.0, df[ax], db[ax]);
    }
    const bool neg = mask[c];
    const double gn = godunov_norm(neg, df[0], db[0], df[1], db[1], df[2], db[2]);
    step[c] = (gn - 1) * __ldg(deltat + c) * (neg ? -1. : 1.);
}

// upwind_normal (ENORK2, enork2_extend.cu:103-141).
__global__ void __launch_bounds__(BX *BY) k_enork2_upwind_normal(Fields6 n, const double *__restrict__ lsf, CFields6 d,
                                                                   Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7];
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        n.p[ax][c] = eno2_upwind(p, __ldg(d.p[2 * ax] + c), __ldg(d.p[2 * ax + 1] + c), axis_h(g, ax));
    }
}

// boundary_interpolate (ENORK2, enork2_extend.cu:175-211): every entry is written.
__global__ void __launch_bounds__(BX *BY) k_enork2_boundary_interpolate(Fields6 cp, CFields6 d,
                                                                          const double *__restrict__ lsf, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7], cf, cb;
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        eno2_crossing(p, __ldg(d.p[2 * ax] + c), __ldg(d.p[2 * ax + 1] + c), axis_h(g, ax), cf, cb);
        cp.p[2 * ax][c] = cf;
        cp.p[2 * ax + 1][c] = cb;
    }
}

// extend_step (ENORK2, enork2_extend.cu:214-267): no fixed-node test.
__global__ void __launch_bounds__(BX *BY) k_enork2_extend_step(double *__restrict__ step,
                                                                 const double *__restrict__ deltat,
                                                                 const double *__restrict__ lsf, CFields6 v3,
                                                                 CFields6 d, CFields6 cp, Grid g)
{
    int i, j, k;
    if (!node_of_thread(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    double df[3], db[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        double p[7];
        load_line7(lsf, axis_line(g, i, j, k, ax), p);
        eno2_pair(p, __ldg(d.p[2 * ax] + c), __ldg(d.p[2 * ax + 1] + c), axis_h(g, ax), __ldg(cp.p[2 * ax] + c),
                  __ldg(cp.p[2 * ax + 1] + c), df[ax], db[ax]);
    }
    step[c] = upwind_dot(__ldg(v3.p[0] + c), __ldg(v3.p[1] + c), __ldg(v3.p[2] + c), df[0], db[0], df[1], db[1],
                         df[2], db[2]) *
              __ldg(deltat + c);
}

// ---- argument checks ---------------------------------------------------------------

template <typename... P> bool any_null(P... p) { return ((p == nullptr) || ...); }

int prologue(int rows, int cols, int pges, double dx, double dy, double dz, long long num_ele, bool check_num)
{
    int st = check_grid(rows, cols, pges, dx, dy, dz);
    if (st) return st;
    if (check_num && (long long)rows * cols * pges != num_ele) return VSL_ERR_SHAPE;
    return VSL_OK;
}

}  // namespace
}  // namespace vsl

using namespace vsl;

extern "C" {

int vsl_boundary_location(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                          const double *lsf, int num_ele, int rows, int cols, int pges, double dx, double dy,
                          double dz, vsl_stream_t stream)
{
    if (any_null(xpr, xpl, ypf, ypb, zpu, zpd, lsf)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    Fields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    k_boundary_location<true><<<node_grid(g), dim3(BX, BY), 0, stream>>>(d, lsf, g);
    return launch_status(cudaGetLastError());
}

int vsl_cubic_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                                  const double *lsf, int num_ele, int rows, int cols, int pges, double dx,
                                  double dy, double dz, vsl_stream_t stream)
{
    if (any_null(xpr, xpl, ypf, ypb, zpu, zpd, lsf)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    Fields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    k_boundary_location<false><<<node_grid(g), dim3(BX, BY), 0, stream>>>(d, lsf, g);
    return launch_status(cudaGetLastError());
}

static int re_step_common(bool eno3, double *step, const double *lsf, const bool *mask, const double *deltat,
                          const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                          const double *zpu, const double *zpd, int rows, int cols, int pges, double dx, double dy,
                          double dz, int num_ele, vsl_stream_t stream)
{
    if (any_null(step, lsf, mask, deltat, xpr, xpl, ypf, ypb, zpu, zpd)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    CFields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    if (eno3)
        k_re_step<true><<<node_grid(g), dim3(BX, BY), 0, stream>>>(step, lsf, mask, deltat, d, g);
    else
        k_re_step<false><<<node_grid(g), dim3(BX, BY), 0, stream>>>(step, lsf, mask, deltat, d, g);
    return launch_status(cudaGetLastError());
}

int vsl_re_step(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                const double *xpl, const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                int rows, int cols, int pges, double dx, double dy, double dz, int num_ele, vsl_stream_t stream)
{
    return re_step_common(false, step, lsf, mask, deltat, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy,
                          dz, num_ele, stream);
}

int vsl_re_step_eno3(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                     const double *xpl, const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                     int rows, int cols, int pges, double dx, double dy, double dz, int num_ele,
                     vsl_stream_t stream)
{
    return re_step_common(true, step, lsf, mask, deltat, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy,
                          dz, num_ele, stream);
}

static int upwind_normal_common(bool eno3, double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                                const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                                const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                                int num_ele, vsl_stream_t stream)
{
    if (any_null(nx, ny, nz, lsf, xpr, xpl, ypf, ypb, zpu, zpd)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    Fields6 n = {{nx, ny, nz, nullptr, nullptr, nullptr}};
    CFields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    if (eno3)
        k_upwind_normal<true><<<node_grid(g), dim3(BX, BY), 0, stream>>>(n, lsf, d, g);
    else
        k_upwind_normal<false><<<node_grid(g), dim3(BX, BY), 0, stream>>>(n, lsf, d, g);
    return launch_status(cudaGetLastError());
}

int vsl_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr, const double *xpl,
                      const double *ypf, const double *ypb, const double *zpu, const double *zpd, int rows, int cols,
                      int pges, double dx, double dy, double dz, int num_ele, vsl_stream_t stream)
{
    return upwind_normal_common(false, nx, ny, nz, lsf, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz,
                                num_ele, stream);
}

int vsl_upwind_normal_eno3(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                           const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                           const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                           int num_ele, vsl_stream_t stream)
{
    return upwind_normal_common(true, nx, ny, nz, lsf, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz,
                                num_ele, stream);
}

static int crossing_common(bool cubic, double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                           const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                           const double *zpu, const double *zpd, const double *lsf, int rows, int cols, int pges,
                           double dx, double dy, double dz, int num_ele, vsl_stream_t stream)
{
    if (any_null(cpr, cpl, cpf, cpb, cpu, cpd, xpr, xpl, ypf, ypb, zpu, zpd, lsf)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    Fields6 cp = {{cpr, cpl, cpf, cpb, cpu, cpd}};
    CFields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    if (cubic)
        k_crossing_plain<true><<<node_grid(g), dim3(BX, BY), 0, stream>>>(cp, d, lsf, g);
    else
        k_crossing_plain<false><<<node_grid(g), dim3(BX, BY), 0, stream>>>(cp, d, lsf, g);
    return launch_status(cudaGetLastError());
}

int vsl_boundary_interpolant(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                             const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                             const double *zpu, const double *zpd, const double *lsf, int rows, int cols, int pges,
                             double dx, double dy, double dz, int num_ele, vsl_stream_t stream)
{
    return crossing_common(false, cpr, cpl, cpf, cpb, cpu, cpd, xpr, xpl, ypf, ypb, zpu, zpd, lsf, rows, cols,
                           pges, dx, dy, dz, num_ele, stream);
}

int vsl_boundary_interpolate_eno3(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                                  const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                  const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                                  int pges, double dx, double dy, double dz, int num_ele, vsl_stream_t stream)
{
    return crossing_common(true, cpr, cpl, cpf, cpb, cpu, cpd, xpr, xpl, ypf, ypb, zpu, zpd, lsf, rows, cols, pges,
                           dx, dy, dz, num_ele, stream);
}

static int extend_step_common(bool eno3, double *step, const double *deltat, const double *lsf, const double *vx,
                              const double *vy, const double *vz, const double *xpr, const double *xpl,
                              const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                              const double *cpr, const double *cpl, const double *cpf, const double *cpb,
                              const double *cpu, const double *cpd, int rows, int cols, int pges, double dx,
                              double dy, double dz, int num_ele, vsl_stream_t stream)
{
    if (any_null(step, deltat, lsf, vx, vy, vz, xpr, xpl, ypf, ypb, zpu, zpd, cpr, cpl, cpf, cpb, cpu, cpd))
        return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    CFields6 v = {{vx, vy, vz, nullptr, nullptr, nullptr}};
    CFields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    CFields6 cp = {{cpr, cpl, cpf, cpb, cpu, cpd}};
    if (eno3)
        k_extend_step<true><<<node_grid(g), dim3(BX, BY), 0, stream>>>(step, deltat, lsf, v, d, cp, g);
    else
        k_extend_step<false><<<node_grid(g), dim3(BX, BY), 0, stream>>>(step, deltat, lsf, v, d, cp, g);
    return launch_status(cudaGetLastError());
}

int vsl_extend_step(double *step, const double *deltat, const double *lsf, const double *vx, const double *vy,
                    const double *vz, const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                    const double *zpu, const double *zpd, const double *cpr, const double *cpl, const double *cpf,
                    const double *cpb, const double *cpu, const double *cpd, int rows, int cols, int pges,
                    double dx, double dy, double dz, int num_ele, vsl_stream_t stream)
{
    return extend_step_common(false, step, deltat, lsf, vx, vy, vz, xpr, xpl, ypf, ypb, zpu, zpd, cpr, cpl, cpf,
                              cpb, cpu, cpd, rows, cols, pges, dx, dy, dz, num_ele, stream);
}

int vsl_extend_step_eno3(double *step, const double *deltat, const double *lsf, const double *vx, const double *vy,
                         const double *vz, const double *xpr, const double *xpl, const double *ypf,
                         const double *ypb, const double *zpu, const double *zpd, const double *cpr,
                         const double *cpl, const double *cpf, const double *cpb, const double *cpu,
                         const double *cpd, int rows, int cols, int pges, double dx, double dy, double dz,
                         int num_ele, vsl_stream_t stream)
{
    return extend_step_common(true, step, deltat, lsf, vx, vy, vz, xpr, xpl, ypf, ypb, zpu, zpd, cpr, cpl, cpf,
                              cpb, cpu, cpd, rows, cols, pges, dx, dy, dz, num_ele, stream);
}

int vsl_enork2_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                                   const double *lsf, int num_ele, int rows, int cols, int pges, double dx,
                                   double dy, double dz, vsl_stream_t stream)
{
    if (any_null(xpr, xpl, ypf, ypb, zpu, zpd, lsf)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    Fields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    k_enork2_boundary_correction<<<node_grid(g), dim3(BX, BY), 0, stream>>>(d, lsf, g);
    return launch_status(cudaGetLastError());
}

int vsl_enork2_re_step(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                       const double *xpl, const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                       int rows, int cols, int pges, double dx, double dy, double dz, int num_ele,
                       vsl_stream_t stream)
{
    if (any_null(step, lsf, mask, deltat, xpr, xpl, ypf, ypb, zpu, zpd)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    CFields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    k_enork2_re_step<<<node_grid(g), dim3(BX, BY), 0, stream>>>(step, lsf, mask, deltat, d, g);
    return launch_status(cudaGetLastError());
}

int vsl_enork2_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                             const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                             const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                             int num_ele, vsl_stream_t stream)
{
    if (any_null(nx, ny, nz, lsf, xpr, xpl, ypf, ypb, zpu, zpd)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    Fields6 n = {{nx, ny, nz, nullptr, nullptr, nullptr}};
    CFields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    k_enork2_upwind_normal<<<node_grid(g), dim3(BX, BY), 0, stream>>>(n, lsf, d, g);
    return launch_status(cudaGetLastError());
}

int vsl_enork2_boundary_interpolate(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                                    const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                    const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                                    int pges, double dx, double dy, double dz, int num_ele, vsl_stream_t stream)
{
    if (any_null(cpr, cpl, cpf, cpb, cpu, cpd, xpr, xpl, ypf, ypb, zpu, zpd, lsf)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    Fields6 cp = {{cpr, cpl, cpf, cpb, cpu, cpd}};
    CFields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    k_enork2_boundary_interpolate<<<node_grid(g), dim3(BX, BY), 0, stream>>>(cp, d, lsf, g);
    return launch_status(cudaGetLastError());
}

int vsl_enork2_extend_step(double *step, const double *deltat, const double *lsf, const double *vx, const double *vy,
                           const double *vz, const double *xpr, const double *xpl, const double *ypf,
                           const double *ypb, const double *zpu, const double *zpd, const double *cpr,
                           const double *cpl, const double *cpf, const double *cpb, const double *cpu,
                           const double *cpd, int rows, int cols, int pges, double dx, double dy, double dz,
                           int num_ele, vsl_stream_t stream)
{
    if (any_null(step, deltat, lsf, vx, vy, vz, xpr, xpl, ypf, ypb, zpu, zpd, cpr, cpl, cpf, cpb, cpu, cpd))
        return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    CFields6 v = {{vx, vy, vz, nullptr, nullptr, nullptr}};
    CFields6 d = {{xpr, xpl, ypf, ypb, zpu, zpd}};
    CFields6 cp = {{cpr, cpl, cpf, cpb, cpu, cpd}};
    k_enork2_extend_step<<<node_grid(g), dim3(BX, BY), 0, stream>>>(step, deltat, lsf, v, d, cp, g);
    return launch_status(cudaGetLastError());
}

int vsl_set_calculus_toolbox(double *Fx, double *Fy, double *Fz, double *FGradMag, double *Nx, double *Ny,
                             double *Nz, double *Fxx, double *Fyy, double *Fzz, double *Fxy, double *Fyz,
                             double *Fzx, double *FLaplacian, double *MeanCurvature, double *GaussianCurvature,
                             double *Heaviside, double *DiracDelta, const double *lsf, const double *HPrimal,
                             int rows, int cols, int pges, double dx, double dy, double dz, double ds, int num_ele,
                             vsl_stream_t stream)
{
    if (any_null(Fx, Fy, Fz, FGradMag, Nx, Ny, Nz, Fxx, Fyy, Fzz, Fxy, Fyz, Fzx, FLaplacian, MeanCurvature,
                 GaussianCurvature, Heaviside, DiracDelta, lsf, HPrimal))
        return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    if (!(ds > 0)) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    Fields18 o = {{Fx, Fy, Fz, FGradMag, Nx, Ny, Nz, Fxx, Fyy, Fzz, Fxy, Fyz, Fzx, FLaplacian, MeanCurvature,
                   GaussianCurvature, Heaviside, DiracDelta}};
    k_set_calculus_toolbox<<<node_grid(g), dim3(BX, BY), 0, stream>>>(o, lsf, HPrimal, g, ds);
    return launch_status(cudaGetLastError());
}

int vsl_auxi_set_calculus_toolbox(
    double *Ax, double *Ay, double *Az, double *AGradMag, double *Cx, double *Cy, double *Cz, double *NormCrossAF,
    double *tx, double *ty, double *tz, double *nx, double *ny, double *nz, double *Axx, double *Ayy, double *Azz,
    double *Axy, double *Ayz, double *Azx, double *ALaplacian, double *GeodesicCurvature, double *NormalCurvature,
    double *GeodesicTorsion, double *BPerpendicular, double *AHeaviside, double *ADiracDelta, const double *lsf,
    const double *AHPrimal, const double *Fx, const double *Fy, const double *Fz, const double *FGradMag,
    const double *Nx, const double *Ny, const double *Nz, const double *Fxx, const double *Fyy, const double *Fzz,
    const double *Fxy, const double *Fyz, const double *Fzx, int rows, int cols, int pges, double dx, double dy,
    double dz, double ds, int num_ele, vsl_stream_t stream)
{
    AuxOut<double> o = {{Ax, Ay, Az, AGradMag, Cx, Cy, Cz, NormCrossAF, tx, ty, tz, nx, ny, nz, Axx, Ayy, Azz, Axy,
                         Ayz, Azx, ALaplacian, GeodesicCurvature, NormalCurvature, GeodesicTorsion, BPerpendicular,
                         AHeaviside, ADiracDelta, nullptr, nullptr}};
    for (int q = 0; q < AUX_OUT_FIELDS - 2; ++q)
        if (o.f[q] == nullptr) return VSL_ERR_NULL;
    AuxFIn<double> fin = {{Fx, Fy, Fz, FGradMag, Nx, Ny, Nz, Fxx, Fyy, Fzz, Fxy, Fyz, Fzx}};
    for (int q = 0; q < 13; ++q)
        if (fin.f[q] == nullptr) return VSL_ERR_NULL;
    if (any_null(lsf, AHPrimal)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, num_ele, true)) return st;
    if (!(ds > 0)) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    return launch_status(launch_auxi_dropin(o, lsf, AHPrimal, fin, g, ds, (cudaStream_t)stream));
}

int vsl_advection_step(double *astep, const double *vx, const double *vy, const double *vz, const double *lsf,
                       int rows, int cols, int pges, double dx, double dy, double dz, vsl_stream_t stream)
{
    if (any_null(astep, vx, vy, vz, lsf)) return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, 0, false)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    CFields6 v = {{vx, vy, vz, nullptr, nullptr, nullptr}};
    k_advection_step<<<node_grid(g), dim3(BX, BY), 0, stream>>>(astep, v, lsf, g);
    return launch_status(cudaGetLastError());
}

int vsl_weno_derivative(double *WENO_back_x, double *WENO_fore_x, double *WENO_back_y, double *WENO_fore_y,
                        double *WENO_back_z, double *WENO_fore_z, const double *lsf, int rows, int cols, int pges,
                        double dx, double dy, double dz, vsl_stream_t stream)
{
    if (any_null(WENO_back_x, WENO_fore_x, WENO_back_y, WENO_fore_y, WENO_back_z, WENO_fore_z, lsf))
        return VSL_ERR_NULL;
    if (int st = prologue(rows, cols, pges, dx, dy, dz, 0, false)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    Fields6 o = {{WENO_back_x, WENO_fore_x, WENO_back_y, WENO_fore_y, WENO_back_z, WENO_fore_z}};
    k_weno_derivative<<<node_grid(g), dim3(BX, BY), 0, stream>>>(o, lsf, g);
    return launch_status(cudaGetLastError());
}

}  // extern "C"
