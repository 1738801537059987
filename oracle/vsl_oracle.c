/*
 * vsl_oracle.c -- CPU restatement of the level-set hot path of the vesicle code.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the tests, the smoke check and the
 * bench's CPU-baseline leg compare against it.  The product (the CUDA library in the
 * package) never links, loads or calls it.
 *
 * Every function restates one reference kernel or device helper (FP64, one "thread" per
 * node, edge-clamped column-major indexing).  Citations are relative to
 * src/7_0_paper/2_0_Vesicle/CUDA_Code/ of the reference repository:
 *   1_3_WENO5RK3_Reinitialization/{shared_utilities.hpp,boundary_location.cu,re_step.cu}
 *   1_1_WENORK3_Reinitialization/weno_rk3_reinitialization.cu
 *   2_2_WENO5RK3_Extend/{shared_utilities.cuh,shared_utilities.cup,upwind_normal.cu,
 *                        boundary_interpolant.cu,extend_step.cu}
 *   2_1_WENORK3_Extend/wenork3_extend.cu
 *   1_0_ENORK2_Reinitialization/boundary_correction.cu, 2_0_ENORK2_Extend/enork2_extend.cu
 *   4_0_Calculus_ToolBox/{set_calculus_toolbox.cu,auxi_set_calculus_toolbox.cu,advection_step.cu}
 *   5_0_Nonoscillating_Reconstruction/nonoscillating_interpolant.cu
 *
 * Arithmetic is kept in the reference's operation order (same association, same
 * constants, same POW() calls) so that, built with -ffp-contract=off, it agrees with the
 * reference compiled for the host to the last bit or within a few ulps.  The grid layout
 * is ind = k*rows*cols + j*rows + i with i = row (y, stride 1), j = column (x), k = page
 * (z); neighbour indices outside the grid are clamped to the edge.
 */
#include <math.h>
#include <stdint.h>
#include <stdbool.h>
#include <string.h>

#include "vsl_oracle.h"

/* The reference calls pow(t, n) for small integer n.  Built with VSL_ORACLE_CR_POW the
 * oracle instead rounds those powers once (the running product kept exactly as a
 * double-double via fma), which is how the CUDA plain form forms them; glibc's pow is
 * accurate to 0.52 ulp but not always correctly rounded, so the two builds can differ in
 * the last bit of a power.  Comparing the CUDA form with the VSL_ORACLE_CR_POW variant
 * isolates everything else to the bit. */
#ifdef VSL_ORACLE_CR_POW
static double cr_pow(double t, double pd)
{
    int n = (int)pd;
    if ((double)n != pd || n < 0 || n > 8) return pow(t, pd);
    if (n == 0) return 1.0;
    if (n == 1) return t;
    double hi = t, lo = 0.0;
    for (int k = 2; k <= n; ++k) {
        double p1 = hi * t;
        double e1 = fma(hi, t, -p1);
        lo = fma(lo, t, e1);
        hi = p1;
    }
    return hi + lo;
}
#define POW cr_pow
#else
#define POW pow
#endif

/* ------------------------------------------------------------------------------------ */
/* indexing                                                                              */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    int rows, cols, pges;
} grid3;

/* Edge clamp of one coordinate: shared_utilities.hpp:21-31 (sub2ind). */
static inline int64_t clampc(int v, int n) { return v < 0 ? 0 : (v > n - 1 ? n - 1 : v); }

static inline int64_t node(const grid3 *g, int i, int j, int k)
{
    return (clampc(k, g->pges) * g->cols + clampc(j, g->cols)) * (int64_t)g->rows + clampc(i, g->rows);
}

enum { AX_X = 0, AX_Y = 1, AX_Z = 2 };

/* node reached from (i,j,k) by s steps along an axis (x = columns, y = rows, z = pages) */
static inline int64_t step_node(const grid3 *g, int i, int j, int k, int axis, int s)
{
    if (axis == AX_X) return node(g, i, j + s, k);
    if (axis == AX_Y) return node(g, i + s, j, k);
    return node(g, i, j, k + s);
}

/* values f[-3..+3] along an axis, clamped (the 7-point line of every WENO kernel) */
static inline void line7(const double *f, const grid3 *g, int i, int j, int k, int axis, double p[7])
{
    for (int s = -3; s <= 3; ++s) p[s + 3] = f[step_node(g, i, j, k, axis, s)];
}

/* ------------------------------------------------------------------------------------ */
/* scalar helpers: shared_utilities.hpp:5-18                                             */
/* ------------------------------------------------------------------------------------ */

static inline double dmax(double x, double y) { return (x < y) ? y : x; }
static inline double dmin(double x, double y) { return (x < y) ? x : y; }
static inline double minmod(double x, double y) { return (x * y < 0) ? 0.0 : (fabs(x) < fabs(y) ? x : y); }
static inline double minabs(double x, double y) { return (fabs(x) < fabs(y)) ? x : y; }
static inline double sgn(double x) { return (x > 0) ? 1.0 : -1.0; }

/* ------------------------------------------------------------------------------------ */
/* Lagrange interpolant in monomial form and Brent root: shared_utilities.hpp:37-173     */
/* ------------------------------------------------------------------------------------ */

/* Monomial coefficients a[0..n] of the degree-n polynomial through (x[m], y[m]), m=0..n.
 * Each Lagrange basis term is expanded by multiplying out its n linear factors in order
 * (coefficients kept highest power first), then the terms are summed per power.
 * Restates Poly<n>::setInterpolation, shared_utilities.hpp:55-103. */
static void lagrange_monomial(int n, const double *x, const double *y, double *a)
{
    double scale[6], roots[6][5], expand[6][6];
    for (int m = 0; m <= n; ++m) {
        scale[m] = y[m];
        int r = 0;
        for (int q = 0; q <= n; ++q) {
            if (q == m) continue;
            scale[m] /= x[m] - x[q];
            roots[m][r++] = x[q];
        }
    }
    for (int m = 0; m <= n; ++m) {
        expand[m][0] = 1.0;
        for (int q = 1; q <= n; ++q) expand[m][q] = 0.0;
        for (int r = 0; r < n; ++r) {
            double nxt[6];
            for (int q = 1; q <= r + 1; ++q) nxt[q] = expand[m][q] - roots[m][r] * expand[m][q - 1];
            for (int q = 1; q <= r + 1; ++q) expand[m][q] = nxt[q];
        }
    }
    for (int p = 0; p <= n; ++p) {
        a[p] = 0.0;
        for (int m = 0; m <= n; ++m) a[p] += scale[m] * expand[m][n - p];
    }
}

/* Poly<n>::operator(), shared_utilities.hpp:47-53: sum of a[p] * POW(t, p). */
static double poly_at(int n, const double *a, double t)
{
    double v = 0;
    for (int p = 0; p <= n; ++p) v += a[p] * POW(t, p);
    return v;
}

/* Brent's method on the polynomial a[0..n] over [x1, x2], tolerance tol, at most 100
 * iterations.  Restates zeroin, shared_utilities.hpp:109-173. */
static double brent_poly(int n, const double *a, double x1, double x2, double tol)
{
    double d = 0, e = 0, p, q, r, s, xm;
    double lo = x1, b = x2, c = x2;
    double flo = poly_at(n, a, lo), fb = poly_at(n, a, b), fc = fb;
    for (int it = 0; it < 100; ++it) {
        if ((fb > 0.0 && fc > 0.0) || (fb < 0.0 && fc < 0.0)) {
            c = lo;
            fc = flo;
            d = b - lo;
            e = d;
        }
        if (fabs(fc) < fabs(fb)) {
            lo = b;
            b = c;
            c = lo;
            flo = fb;
            fb = fc;
            fc = flo;
        }
        xm = 0.5 * (c - b);
        if (fabs(xm) <= tol || fb == 0.0) return b;
        if (fabs(e) < tol || fabs(flo) <= fabs(fb)) {
            d = xm;
            e = xm;
        } else {
            s = fb / flo;
            if (lo == c) {
                p = 2.0 * xm * s;
                q = 1.0 - s;
            } else {
                q = flo / fc;
                r = fb / fc;
                p = s * (2.0 * xm * q * (q - r) - (b - lo) * (r - 1.0));
                q = (q - 1.0) * (r - 1.0) * (s - 1.0);
            }
            if (p > 0) q = -q;
            p = fabs(p);
            double lim1 = 3.0 * xm * q - fabs(tol * q);
            double lim2 = fabs(e * q);
            if (2.0 * p < dmin(lim1, lim2)) {
                e = d;
                d = p / q;
            } else {
                d = xm;
                e = d;
            }
        }
        lo = b;
        flo = fb;
        if (fabs(d) > tol)
            b = b + d;
        else
            b += sgn(xm) * tol;
        fb = poly_at(n, a, b);
    }
    return b;
}

/* ------------------------------------------------------------------------------------ */
/* sub-cell interface distances                                                          */
/* ------------------------------------------------------------------------------------ */

/* Quadratic-ENO distance from node b to the interface between b and c (b*c < 0); a is
 * the node before b, d the node after c.  Restates sp, boundary_location.cu:6-20. */
static double eno2_distance(double a, double b, double c, double d, double h)
{
    double eps = 10e-10;
    double d2l = c - 2.0 * b + a;
    double d2r = d - 2.0 * c + b;
    double d2 = minmod(d2l, d2r);
    if (d2 > eps || d2 < -eps) {
        double disc = POW((0.5 * d2 - b - c), 2) - 4. * b * c;
        return h * (0.5 + (b - c - sgn(b - c) * sqrt(disc)) / d2);
    }
    return (h * b / (b - c));
}

/* Degree-5 distance: samples at 0,h,..,5h, crossing between 2h and 3h.  Falls back to the
 * quadratic ENO distance next to a kink.  Restates six_distance, boundary_location.cu:53-80. */
static double quintic_distance(const double v[6], double h)
{
    if (v[1] * v[2] < 0 || v[3] * v[4] < 0) return eno2_distance(v[1], v[2], v[3], v[4], h);
    double xs[6] = {0.0, h, 2 * h, 3 * h, 4 * h, 5 * h};
    double a[6];
    lagrange_monomial(5, xs, v, a);
    double t = brent_poly(5, a, 2 * h, 3 * h, 3e-16);
    t = dmax(t, 2 * h);
    t = dmin(t, 3 * h);
    return (t - 2 * h);
}

/* Cubic distance with Newton's method: samples at 0,h,2h,3h, crossing between h and 2h.
 * Restates cubic_distance, weno_rk3_reinitialization.cu:73-116. */
static double cubic_newton_distance(double v0, double v1, double v2, double v3, double h)
{
    if (v0 * v1 < 0 || v2 * v3 < 0) return eno2_distance(v0, v1, v2, v3, h);
    double a0 = v0;
    double a1 = (3.0 * (v1 - v0) - 3.0 / 2.0 * (v2 - v0) + 1.0 / 3.0 * (v3 - v0)) / h;
    double a2 = (-5.0 / 2.0 * (v1 - v0) + 2.0 * (v2 - v0) - 1.0 / 2.0 * (v3 - v0)) / POW(h, 2);
    double a3 = (1.0 / 2.0 * (v1 - v0) - 1.0 / 2.0 * (v2 - v0) + 1.0 / 6.0 * (v3 - v0)) / POW(h, 3);
    double t = h + h * v1 / (v1 - v2);
    int it = 0;
    double change = 1;
    while (change > 1e-14 && it < 50) {
        double f = a0 + a1 * t + a2 * t * t + a3 * t * t * t;
        double df = a1 + 2 * a2 * t + 3 * a3 * t * t;
        double tn = t - f / df;
        change = fabs(f / df);
        it++;
        t = tn;
    }
    t = dmax(t, h);
    t = dmin(t, 2 * h);
    return (t - h);
}

/* ------------------------------------------------------------------------------------ */
/* one-sided derivatives                                                                 */
/* ------------------------------------------------------------------------------------ */

/* Jiang-Shu WENO5 one-sided derivative from five consecutive first differences, biased
 * toward the third; weights omega_k = alpha_k/sum formed before the weighted sum.
 * Restates weno_onesided_derivative, re_step.cu:11-37. */
static double weno5_ref_order(double v1, double v2, double v3, double v4, double v5)
{
    double q1 = 1. / 3. * v1 - 7. / 6. * v2 + 11. / 6. * v3;
    double q2 = -1. / 6. * v2 + 5. / 6. * v3 + 1. / 3. * v4;
    double q3 = 1. / 3. * v3 + 5. / 6. * v4 - 1. / 6. * v5;
    double s1 = 13. / 12. * POW((v1 - 2 * v2 + v3), 2) + 1. / 4. * POW((v1 - 4 * v2 + 3 * v3), 2);
    double s2 = 13. / 12. * POW((v2 - 2 * v3 + v4), 2) + 1. / 4. * POW((v2 - v4), 2);
    double s3 = 13. / 12. * POW((v3 - 2 * v4 + v5), 2) + 1. / 4. * POW((3 * v3 - 4 * v4 + v5), 2);
    double eps = 1e-6;
    double a1 = 0.1 / POW((s1 + eps), 2);
    double a2 = 0.6 / POW((s2 + eps), 2);
    double a3 = 0.3 / POW((s3 + eps), 2);
    double tot = a1 + a2 + a3;
    double o1 = a1 / tot, o2 = a2 / tot, o3 = a3 / tot;
    return (o1 * q1 + o2 * q2 + o3 * q3);
}

/* Seven-point stencil with the interface inserted: positions xs[0..6] relative to the
 * centre (xs[3] = 0) and values hs[0..6].  p1..p7 are the node values, r1/l1 the
 * distances from the centre to the interface forward/backward, hf/hb the values the
 * field takes on the interface.  Restates select_stencil, re_step.cu:41-77 (interface
 * value 0) and shared_utilities.cup:211-247 (interface values hf/hb). */
static void insert_interface(const double p[7], double r1, double l1, double h, double hf, double hb,
                             double xs[7], double hs[7])
{
    hs[3] = p[3];
    xs[3] = 0.0;
    if (r1 < h) {
        xs[4] = r1; xs[5] = h; xs[6] = 2 * h;
        hs[4] = hf; hs[5] = p[4]; hs[6] = p[5];
    } else {
        xs[4] = h; xs[5] = 2 * h; xs[6] = 3 * h;
        hs[4] = p[4]; hs[5] = p[5]; hs[6] = p[6];
    }
    if (l1 < h) {
        xs[2] = -l1; xs[1] = -h; xs[0] = -2 * h;
        hs[2] = hb; hs[1] = p[2]; hs[0] = p[1];
    } else {
        xs[2] = -h; xs[1] = -2 * h; xs[0] = -3 * h;
        hs[2] = p[2]; hs[1] = p[1]; hs[0] = p[0];
    }
}

/* Smoothness indicators of the three candidate stencils of the nonuniform WENO
 * reconstruction.  e[0..5] are the cell faces (x_{-2.5} .. x_{2.5} in the reference's
 * naming) and u[0..4] the cell averages (u_{-2} .. u_{2}).  re_step.cu:116-158 and
 * :190-232 (the same expressions serve both biases). */
static void nu_smoothness(const double e[6], const double u[5], double s[3])
{
    double xm25 = e[0], xm15 = e[1], xm05 = e[2], x05 = e[3], x15 = e[4], x25 = e[5];
    double um2 = u[0], um1 = u[1], u0 = u[2], u1 = u[3], u2 = u[4];
    s[0] = 4.0 * POW((x05 - xm05) / (x25 - xm05), 2) *
           (POW((u2 - u1) / (x25 - x05), 2) * (10.0 * POW(x05 - xm05, 2) + (x15 - xm05) * (x15 - x05)) +
            (u2 - u1) * (u0 - u1) / ((x25 - x05) * (x15 - xm05)) *
                (20.0 * POW(x05 - xm05, 2) + 2.0 * (x15 - xm05) * (x15 - x05) + (x25 - xm05) * (2.0 * x15 - x05 - xm05)) +
            POW((u0 - u1) / (x15 - xm05), 2) * (10.0 * POW(x05 - xm05, 2) + (x25 + x15 - 2.0 * xm05) * (x25 + x15 - x05 - xm05)));
    s[1] = 4.0 * POW((x05 - xm05) / (x15 - xm15), 2) *
           (POW((um1 - u0) / (x05 - xm15), 2) * (10.0 * POW(x05 - xm05, 2) + (x15 - xm05) * (x15 - x05)) +
            (u1 - u0) * (um1 - u0) / ((x15 - xm05) * (x05 - xm15)) *
                (20.0 * POW(x05 - xm05, 2) - (x15 - x05) * (xm05 - xm15) - (x15 - xm05) * (x05 - xm15)) +
            POW((u1 - u0) / (x15 - xm05), 2) * (10.0 * POW(x05 - xm05, 2) + (xm05 - xm15) * (x05 - xm15)));
    s[2] = 4.0 * POW((x05 - xm05) / (x05 - xm25), 2) *
           (POW((um2 - um1) / (xm05 - xm25), 2) * (10.0 * POW(x05 - xm05, 2) + (x05 - xm15) * (xm05 - xm15)) +
            (u0 - um1) * (um2 - um1) / ((x05 - xm15) * (xm05 - xm25)) *
                (20.0 * POW(x05 - xm05, 2) + 2.0 * (x05 - xm15) * (xm05 - xm15) + (x05 - xm25) * (x05 + xm05 - 2.0 * xm15)) +
            POW((u0 - um1) / (x05 - xm15), 2) * (10.0 * POW(x05 - xm05, 2) + (2.0 * x05 - xm25 - xm15) * (x05 + xm05 - xm15 - xm25)));
}

static double nu_combine(const double v[3], const double c[3], const double s[3])
{
    double eps = 1e-6;
    double a0 = c[0] / POW((s[0] + eps), 2);
    double a1 = c[1] / POW((s[1] + eps), 2);
    double a2 = c[2] / POW((s[2] + eps), 2);
    double tot = a0 + a1 + a2;
    double o0 = a0 / tot, o1 = a1 / tot, o2 = a2 / tot;
    return v[0] * o0 + v[1] * o1 + v[2] * o2;
}

/* Nonuniform WENO forward/backward derivatives at xs[3] = 0 from a seven-point stencil
 * with arbitrary spacing.  Restates weno_nonuniform, re_step.cu:79-243. */
static void weno_nonuniform_pair(const double xs[7], const double hs[7], double *d_fore, double *d_back)
{
    /* first divided differences on the six cells */
    double dd[6];
    for (int m = 0; m < 6; ++m) dd[m] = (hs[m + 1] - hs[m]) / (xs[m + 1] - xs[m]);
    double e[6], u[5], v[3], c[3], s[3];

    /* forward bias: faces xs[1..6], cells dd[1..5], value at the face xs[3] */
    for (int m = 0; m < 6; ++m) e[m] = xs[m + 1];
    for (int m = 0; m < 5; ++m) u[m] = dd[m + 1];
    {
        double xm25 = e[0], xm15 = e[1], xm05 = e[2], x05 = e[3], x15 = e[4], x25 = e[5];
        double um2 = u[0], um1 = u[1], u0 = u[2], u1 = u[3], u2 = u[4];
        v[0] = u1 + (u0 - u1) * (1.0 + (x05 - xm05) / (x15 - xm05) + (x05 - xm05) / (x25 - xm05)) +
               (u2 - u1) * ((x05 - xm05) / (x25 - xm05)) * ((x15 - xm05) / (x25 - x05));
        v[1] = u0 + (um1 - u0) * ((x05 - xm05) / (x15 - xm15)) * ((x15 - xm05) / (x05 - xm15)) -
               (u1 - u0) * ((x05 - xm05) / (x15 - xm15)) * ((xm05 - xm15) / (x15 - xm05));
        v[2] = um1 + (u0 - um1) * ((xm05 - xm15) / (x05 - xm25)) * ((xm05 - xm25) / (x05 - xm15)) -
               (um2 - um1) * ((xm05 - xm15) / (x05 - xm25)) * ((x05 - xm05) / (xm05 - xm25));
        c[0] = ((xm05 - xm15) / (x25 - xm25)) * ((xm05 - xm25) / (x25 - xm15));
        c[1] = ((xm05 - xm25) / (x25 - xm25)) * ((x25 - xm05) / (x25 - xm15)) * (1.0 + (x25 - xm15) / (x15 - xm25));
        c[2] = ((x15 - xm05) / (x25 - xm25)) * ((x25 - xm05) / (x15 - xm25));
    }
    nu_smoothness(e, u, s);
    *d_fore = nu_combine(v, c, s);

    /* backward bias: faces xs[0..5], cells dd[0..4], value at the face xs[3] */
    for (int m = 0; m < 6; ++m) e[m] = xs[m];
    for (int m = 0; m < 5; ++m) u[m] = dd[m];
    {
        double xm25 = e[0], xm15 = e[1], xm05 = e[2], x05 = e[3], x15 = e[4], x25 = e[5];
        double um2 = u[0], um1 = u[1], u0 = u[2], u1 = u[3], u2 = u[4];
        v[0] = u1 + (u0 - u1) * ((x15 - x05) / (x25 - xm05)) * ((x25 - x05) / (x15 - xm05)) -
               (u2 - u1) * ((x15 - x05) / (x25 - xm05)) * ((x05 - xm05) / (x25 - x05));
        v[1] = u0 + (u1 - u0) * ((x05 - xm05) / (x15 - xm15)) * ((x05 - xm15) / (x15 - xm05)) -
               (um1 - u0) * ((x05 - xm05) / (x15 - xm15)) * ((x15 - x05) / (x05 - xm15));
        v[2] = um1 + (um2 - um1) * ((x05 - xm05) / (xm05 - xm25)) * ((x05 - xm15) / (x05 - xm25)) +
               (u0 - um1) * (1.0 + (x05 - xm05) / (x05 - xm15) + (x05 - xm05) / (x05 - xm25));
        c[0] = ((x05 - xm25) / (x25 - xm25)) * ((x05 - xm15) / (x25 - xm15));
        c[1] = ((x05 - xm25) / (x25 - xm25)) * ((x25 - x05) / (x25 - xm15)) * (1.0 + (x25 - xm15) / (x15 - xm25));
        c[2] = ((x15 - x05) / (x25 - xm25)) * ((x25 - x05) / (x15 - xm25));
    }
    nu_smoothness(e, u, s);
    *d_back = nu_combine(v, c, s);
}

/* Nonuniform cubic ENO forward/backward derivatives at xs[3] = 0 (the "ENO3" scheme).
 * Restates ENO_cubic_derivative, weno_rk3_reinitialization.cu:189-222. */
static void eno3_nonuniform_pair(const double xs[7], const double hs[7], double *d_fore, double *d_back)
{
    double x3m = xs[0], x2m = xs[1], x1m = xs[2], x0 = xs[3], x1 = xs[4], x2 = xs[5], x3 = xs[6];
    double h3m = hs[0], h2m = hs[1], h1m = hs[2], h0 = hs[3], h1 = hs[4], h2 = hs[5], h3 = hs[6];
    double f25 = (h3 - h2) / (x3 - x2);
    double f15 = (h2 - h1) / (x2 - x1);
    double f05 = (h1 - h0) / (x1 - x0);
    double fm05 = (h0 - h1m) / (x0 - x1m);
    double fm15 = (h1m - h2m) / (x1m - x2m);
    double fm25 = (h2m - h3m) / (x2m - x3m);

    double g2 = (f25 - f15) / (x3 - x1);
    double g1 = (f15 - f05) / (x2 - x0);
    double g0 = (f05 - fm05) / (x1 - x1m);
    double gm1 = (fm05 - fm15) / (x0 - x2m);
    double gm2 = (fm15 - fm25) / (x1m - x3m);

    double t15 = (g2 - g1) / (x3 - x0);
    double t05 = (g1 - g0) / (x2 - x1m);
    double tm05 = (g0 - gm1) / (x1 - x2m);
    double tm15 = (gm1 - gm2) / (x0 - x3m);

    double a1 = (x0 - x1m) * (x0 - x2m) * minabs(tm05, tm15);
    double a2 = (x0 - x1m) * (x0 - x1) * minabs(tm05, t05);
    double a = (fabs(gm1) < fabs(g0)) ? a1 : a2;
    double b1 = (x0 - x1m) * (x0 - x1) * minabs(tm05, t05);
    double b2 = (x0 - x1) * (x0 - x2) * minabs(t05, t15);
    double b = (fabs(g0) < fabs(g1)) ? b1 : b2;

    *d_back = fm05 + minmod(gm1, g0) * (x0 - x1m) + a;
    *d_fore = f05 + minmod(g0, g1) * (x0 - x1) + b;
}

/* Choice between the uniform WENO5 derivatives and the interface-aware nonuniform ones.
 *   trigger_on_sign: reinitialization (re_step.cu:248-269): p3*p4<0 || p4*p5<0;
 *   otherwise extension/normals (shared_utilities.cup:418-440): r1<h || l1<h.
 *   eno3 selects ENO_cubic_derivative (weno_rk3_reinitialization.cu:227-248,
 *   wenork3_extend.cu:166-188) instead of the nonuniform WENO. */
static void axis_derivatives(const double p[7], double r1, double l1, double h, double hf, double hb,
                             int trigger_on_sign, int eno3, double *d_fore, double *d_back)
{
    int near;
    if (trigger_on_sign)
        near = p[2] * p[3] < 0 || p[3] * p[4] < 0;
    else
        near = r1 < h || l1 < h;
    if (near) {
        double xs[7], hs[7];
        insert_interface(p, r1, l1, h, hf, hb, xs, hs);
        if (eno3)
            eno3_nonuniform_pair(xs, hs, d_fore, d_back);
        else
            weno_nonuniform_pair(xs, hs, d_fore, d_back);
    } else {
        double v[6];
        for (int m = 0; m < 6; ++m) v[m] = (p[m + 1] - p[m]) / h;
        *d_back = weno5_ref_order(v[0], v[1], v[2], v[3], v[4]);
        *d_fore = weno5_ref_order(v[5], v[4], v[3], v[2], v[1]);
    }
}

/* ------------------------------------------------------------------------------------ */
/* kernels (one loop iteration = one reference thread)                                   */
/* ------------------------------------------------------------------------------------ */

#define FOR_EACH_NODE(g)                                         \
    _Pragma("omp parallel for schedule(static)")                 \
    for (int k = 0; k < (g).pges; ++k)                           \
        for (int j = 0; j < (g).cols; ++j)                       \
            for (int i = 0; i < (g).rows; ++i)

/* boundary_location (WENO5) and boundary_correction (ENO3): the distance from each node
 * to an interface crossing the +x/+y/+z grid edge; scatter form with the reference's
 * in/out semantics (entries without a crossing keep the caller's value).
 * boundary_location.cu:84-132; weno_rk3_reinitialization.cu:251-293. */
static void distances_impl(double *fore[3], double *back[3], const double *f, grid3 g, const double h[3], int quintic)
{
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        double f0 = f[c];
        for (int ax = 0; ax < 3; ++ax) {
            int64_t nb = step_node(&g, i, j, k, ax, 1);
            double f2 = f[nb];
            if (!(f0 * f2 < 0)) continue;
            double dist;
            if (quintic) {
                double v[6];
                for (int s = -2; s <= 3; ++s) v[s + 2] = f[step_node(&g, i, j, k, ax, s)];
                dist = quintic_distance(v, h[ax]);
            } else {
                dist = cubic_newton_distance(f[step_node(&g, i, j, k, ax, -1)], f0, f2,
                                             f[step_node(&g, i, j, k, ax, 2)], h[ax]);
            }
            fore[ax][c] = dist;
            back[ax][nb] = h[ax] - fore[ax][c];
        }
    }
}

void orc_boundary_location(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                           const double *lsf, int num_ele, int rows, int cols, int pges, double dx, double dy,
                           double dz)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    distances_impl(fore, back, lsf, g, h, 1);
}

void orc_cubic_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                                   const double *lsf, int num_ele, int rows, int cols, int pges, double dx,
                                   double dy, double dz)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    distances_impl(fore, back, lsf, g, h, 0);
}

/* re_step (WENO5, re_step.cu:283-393) and re_step (ENO3, weno_rk3_reinitialization.cu:
 * 295-406): Godunov Hamiltonian of |grad phi| - 1 times dt, sign from the mask. */
static void re_step_impl(double *step, const double *lsf, const bool *mask, const double *deltat,
                         const double *fore[3], const double *back[3], grid3 g, const double h[3], int eno3)
{
    double tiny = 1e-6 * h[0];
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        if (fore[0][c] < tiny || back[0][c] < tiny || fore[1][c] < tiny || back[1][c] < tiny ||
            fore[2][c] < tiny || back[2][c] < tiny) {
            step[c] = 0;
            continue;
        }
        double df[3], db[3];
        for (int ax = 0; ax < 3; ++ax) {
            double p[7];
            line7(lsf, &g, i, j, k, ax, p);
            axis_derivatives(p, fore[ax][c], back[ax][c], h[ax], 0.0, 0.0, 1, eno3, &df[ax], &db[ax]);
        }
        double xR = df[0], xL = db[0], yF = df[1], yB = db[1], zU = df[2], zD = db[2];
        if (mask[c]) {
            step[c] = (sqrt(dmax(POW(dmin(0.0, xL), 2), POW(dmax(0.0, xR), 2)) +
                            dmax(POW(dmin(0.0, yB), 2), POW(dmax(0.0, yF), 2)) +
                            dmax(POW(dmin(0.0, zD), 2), POW(dmax(0.0, zU), 2))) - 1) * deltat[c] * (-1.);
        } else {
            step[c] = (sqrt(dmax(POW(dmax(0.0, xL), 2), POW(dmin(0.0, xR), 2)) +
                            dmax(POW(dmax(0.0, yB), 2), POW(dmin(0.0, yF), 2)) +
                            dmax(POW(dmax(0.0, zD), 2), POW(dmin(0.0, zU), 2))) - 1) * deltat[c] * (1.);
        }
    }
}

void orc_re_step(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                 const double *xpl, const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                 int rows, int cols, int pges, double dx, double dy, double dz, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    re_step_impl(step, lsf, mask, deltat, fore, back, g, h, 0);
}

void orc_re_step_eno3(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                      const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                      const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                      int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    re_step_impl(step, lsf, mask, deltat, fore, back, g, h, 1);
}

/* upwind_normal (upwind_normal.cu:4-104; wenork3_extend.cu:192-292): per axis the
 * one-sided derivative taken toward the neighbour of smaller |phi|. */
static void upwind_normal_impl(double *n[3], const double *lsf, const double *fore[3], const double *back[3],
                               grid3 g, const double h[3], int eno3)
{
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        for (int ax = 0; ax < 3; ++ax) {
            double p[7], df, db;
            line7(lsf, &g, i, j, k, ax, p);
            axis_derivatives(p, fore[ax][c], back[ax][c], h[ax], 0.0, 0.0, 0, eno3, &df, &db);
            n[ax][c] = (fabs(p[4]) < fabs(p[2])) ? df : db;
        }
    }
}

void orc_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr, const double *xpl,
                       const double *ypf, const double *ypb, const double *zpu, const double *zpd, int rows,
                       int cols, int pges, double dx, double dy, double dz, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    double *n[3] = {nx, ny, nz};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    upwind_normal_impl(n, lsf, fore, back, g, h, 0);
}

void orc_upwind_normal_eno3(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                            const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                            const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                            int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    double *n[3] = {nx, ny, nz};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    upwind_normal_impl(n, lsf, fore, back, g, h, 1);
}

/* Value of the field on the interface crossing, from the degree-5 interpolant through
 * the six nodes around it (sixth_interp, boundary_interpolant.cu:78-99), or from the
 * cubic through four nodes (cubic_interp, wenork3_extend.cu:296-328).  0 where the
 * distance says there is no crossing. */
static void crossing_values_quintic(const double p[7], double dis_f, double dis_b, double h, double *cf, double *cb)
{
    *cf = 0.0;
    *cb = 0.0;
    if (dis_f < h) {
        double xs[6] = {h, 2 * h, 3 * h, 4 * h, 5 * h, 6 * h};
        double a[6];
        lagrange_monomial(5, xs, p + 1, a);
        *cf = poly_at(5, a, 3 * h + dis_f);
    }
    if (dis_b < h) {
        double xs[6] = {0.0, h, 2 * h, 3 * h, 4 * h, 5 * h};
        double a[6];
        lagrange_monomial(5, xs, p, a);
        *cb = poly_at(5, a, 3 * h - dis_b);
    }
}

static void cubic_coefficients(double v0, double v1, double v2, double v3, double h, double a[4])
{
    a[0] = v0;
    a[1] = (3.0 * (v1 - v0) - 3.0 / 2.0 * (v2 - v0) + 1.0 / 3.0 * (v3 - v0)) / h;
    a[2] = (-5.0 / 2.0 * (v1 - v0) + 2.0 * (v2 - v0) - 1.0 / 2.0 * (v3 - v0)) / POW(h, 2);
    a[3] = (1.0 / 2.0 * (v1 - v0) - 1.0 / 2.0 * (v2 - v0) + 1.0 / 6.0 * (v3 - v0)) / POW(h, 3);
}

static void crossing_values_cubic(const double p[7], double dis_f, double dis_b, double h, double *cf, double *cb)
{
    *cf = 0.;
    *cb = 0.;
    double a[4];
    if (dis_f < h) {
        cubic_coefficients(p[2], p[3], p[4], p[5], h, a);
        double t = h + dis_f;
        *cf = a[0] + a[1] * t + a[2] * POW(t, 2) + a[3] * POW(t, 3);
    }
    if (dis_b < h) {
        cubic_coefficients(p[1], p[2], p[3], p[4], h, a);
        double t = 2 * h - dis_b;
        *cb = a[0] + a[1] * t + a[2] * POW(t, 2) + a[3] * POW(t, 3);
    }
}

static void crossing_impl(double *cf[3], double *cb[3], const double *fore[3], const double *back[3],
                          const double *lsf, grid3 g, const double h[3], int cubic)
{
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        for (int ax = 0; ax < 3; ++ax) {
            double p[7];
            line7(lsf, &g, i, j, k, ax, p);
            if (cubic)
                crossing_values_cubic(p, fore[ax][c], back[ax][c], h[ax], &cf[ax][c], &cb[ax][c]);
            else
                crossing_values_quintic(p, fore[ax][c], back[ax][c], h[ax], &cf[ax][c], &cb[ax][c]);
        }
    }
}

void orc_boundary_interpolant(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                              const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                              const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                              int pges, double dx, double dy, double dz, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    double *cf[3] = {cpr, cpf, cpu}, *cb[3] = {cpl, cpb, cpd};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    crossing_impl(cf, cb, fore, back, lsf, g, h, 0);
}

void orc_boundary_interpolate_eno3(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                                   const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                   const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                                   int pges, double dx, double dy, double dz, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    double *cf[3] = {cpr, cpf, cpu}, *cb[3] = {cpl, cpb, cpd};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    crossing_impl(cf, cb, fore, back, lsf, g, h, 1);
}

/* extend_step (extend_step.cu:10-125; wenork3_extend.cu:372-487): upwind transport of
 * the field along v with the interface-aware derivatives; fixed nodes step 0. */
static void extend_step_impl(double *step, const double *deltat, const double *lsf, const double *v[3],
                             const double *fore[3], const double *back[3], const double *cf[3],
                             const double *cb[3], grid3 g, const double h[3], int eno3)
{
    double tiny = 1e-6 * h[0];
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        if (fore[0][c] < tiny || back[0][c] < tiny || fore[1][c] < tiny || back[1][c] < tiny ||
            fore[2][c] < tiny || back[2][c] < tiny) {
            step[c] = 0;
            continue;
        }
        double df[3], db[3];
        for (int ax = 0; ax < 3; ++ax) {
            double p[7];
            line7(lsf, &g, i, j, k, ax, p);
            axis_derivatives(p, fore[ax][c], back[ax][c], h[ax], cf[ax][c], cb[ax][c], 0, eno3, &df[ax], &db[ax]);
        }
        step[c] = (dmin(0.0, v[0][c]) * df[0] + dmax(0.0, v[0][c]) * db[0] + dmin(0.0, v[1][c]) * df[1] +
                   dmax(0.0, v[1][c]) * db[1] + dmin(0.0, v[2][c]) * df[2] + dmax(0.0, v[2][c]) * db[2]) *
                  deltat[c];
    }
}

void orc_extend_step(double *step, const double *deltat, const double *lsf, const double *vx, const double *vy,
                     const double *vz, const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                     const double *zpu, const double *zpd, const double *cpr, const double *cpl,
                     const double *cpf, const double *cpb, const double *cpu, const double *cpd, int rows,
                     int cols, int pges, double dx, double dy, double dz, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    const double *v[3] = {vx, vy, vz};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    const double *cf[3] = {cpr, cpf, cpu}, *cb[3] = {cpl, cpb, cpd};
    double h[3] = {dx, dy, dz};
    extend_step_impl(step, deltat, lsf, v, fore, back, cf, cb, g, h, 0);
}

void orc_extend_step_eno3(double *step, const double *deltat, const double *lsf, const double *vx,
                          const double *vy, const double *vz, const double *xpr, const double *xpl,
                          const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                          const double *cpr, const double *cpl, const double *cpf, const double *cpb,
                          const double *cpu, const double *cpd, int rows, int cols, int pges, double dx, double dy,
                          double dz, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    const double *v[3] = {vx, vy, vz};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    const double *cf[3] = {cpr, cpf, cpu}, *cb[3] = {cpl, cpb, cpd};
    double h[3] = {dx, dy, dz};
    extend_step_impl(step, deltat, lsf, v, fore, back, cf, cb, g, h, 1);
}

/* advection_step (advection_step.cu:10-56): upwind WENO5 v.grad(phi), no time step. */
void orc_advection_step(double *astep, const double *vx, const double *vy, const double *vz, const double *lsf,
                        int rows, int cols, int pges, double dx, double dy, double dz)
{
    grid3 g = {rows, cols, pges};
    double h[3] = {dx, dy, dz};
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        double df[3], db[3];
        for (int ax = 0; ax < 3; ++ax) {
            double p[7], v[6];
            line7(lsf, &g, i, j, k, ax, p);
            for (int m = 0; m < 6; ++m) v[m] = (p[m + 1] - p[m]) / h[ax];
            db[ax] = weno5_ref_order(v[0], v[1], v[2], v[3], v[4]);
            df[ax] = weno5_ref_order(v[5], v[4], v[3], v[2], v[1]);
        }
        astep[c] = (dmin(0.0, vx[c]) * df[0] + dmax(0.0, vx[c]) * db[0] + dmin(0.0, vy[c]) * df[1] +
                    dmax(0.0, vy[c]) * db[1] + dmin(0.0, vz[c]) * df[2] + dmax(0.0, vz[c]) * db[2]);
    }
}

/* weno_derivative (nonoscillating_interpolant.cu:59-122): the six one-sided WENO5
 * derivatives as separate fields. */
void orc_weno_derivative(double *back_x, double *fore_x, double *back_y, double *fore_y, double *back_z,
                         double *fore_z, const double *lsf, int rows, int cols, int pges, double dx, double dy,
                         double dz)
{
    grid3 g = {rows, cols, pges};
    double h[3] = {dx, dy, dz};
    double *bk[3] = {back_x, back_y, back_z}, *fr[3] = {fore_x, fore_y, fore_z};
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        for (int ax = 0; ax < 3; ++ax) {
            double p[7], v[6];
            line7(lsf, &g, i, j, k, ax, p);
            for (int m = 0; m < 6; ++m) v[m] = (p[m + 1] - p[m]) / h[ax];
            bk[ax][c] = weno5_ref_order(v[0], v[1], v[2], v[3], v[4]);
            fr[ax][c] = weno5_ref_order(v[5], v[4], v[3], v[2], v[1]);
        }
    }
}

/* set_calculus_toolbox (set_calculus_toolbox.cu:9-107): central-difference gradient,
 * Hessian, curvatures and the Heaviside/Dirac functions from the primal HP = max(phi,0). */
void orc_set_calculus_toolbox(double *Fx, double *Fy, double *Fz, double *FGradMag, double *Nx, double *Ny,
                              double *Nz, double *Fxx, double *Fyy, double *Fzz, double *Fxy, double *Fyz,
                              double *Fzx, double *FLaplacian, double *MeanCurvature, double *GaussianCurvature,
                              double *Heaviside, double *DiracDelta, const double *lsf, const double *HPrimal,
                              int rows, int cols, int pges, double dx, double dy, double dz, double ds, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        int64_t xp = node(&g, i, j + 1, k), xm = node(&g, i, j - 1, k);
        int64_t yp = node(&g, i + 1, j, k), ym = node(&g, i - 1, j, k);
        int64_t zp = node(&g, i, j, k + 1), zm = node(&g, i, j, k - 1);
        double fx = (lsf[xp] - lsf[xm]) / (2 * dx);
        double fy = (lsf[yp] - lsf[ym]) / (2 * dy);
        double fz = (lsf[zp] - lsf[zm]) / (2 * dz);
        double gm = sqrt(fx * fx + fy * fy + fz * fz);
        gm = dmax(gm, 1e-14);
        Fx[c] = fx;
        Fy[c] = fy;
        Fz[c] = fz;
        FGradMag[c] = gm;
        Nx[c] = fx / gm;
        Ny[c] = fy / gm;
        Nz[c] = fz / gm;

        double fxx = (lsf[xp] - 2 * lsf[c] + lsf[xm]) / (dx * dx);
        double fyy = (lsf[yp] - 2 * lsf[c] + lsf[ym]) / (dy * dy);
        double fzz = (lsf[zp] - 2 * lsf[c] + lsf[zm]) / (dz * dz);
        double fxy = (lsf[node(&g, i + 1, j + 1, k)] + lsf[node(&g, i - 1, j - 1, k)] - lsf[node(&g, i + 1, j - 1, k)] -
                      lsf[node(&g, i - 1, j + 1, k)]) / (4 * ds * ds);
        double fyz = (lsf[node(&g, i + 1, j, k + 1)] + lsf[node(&g, i - 1, j, k - 1)] - lsf[node(&g, i + 1, j, k - 1)] -
                      lsf[node(&g, i - 1, j, k + 1)]) / (4 * ds * ds);
        double fzx = (lsf[node(&g, i, j + 1, k + 1)] + lsf[node(&g, i, j - 1, k - 1)] - lsf[node(&g, i, j + 1, k - 1)] -
                      lsf[node(&g, i, j - 1, k + 1)]) / (4 * ds * ds);
        double lap = fxx + fyy + fzz;
        Fxx[c] = fxx;
        Fyy[c] = fyy;
        Fzz[c] = fzz;
        Fxy[c] = fxy;
        Fyz[c] = fyz;
        Fzx[c] = fzx;
        FLaplacian[c] = lap;

        double r1 = fxx * fx + fxy * fy + fzx * fz;
        double r2 = fxy * fx + fyy * fy + fyz * fz;
        double r3 = fzx * fx + fyz * fy + fzz * fz;
        MeanCurvature[c] = -lap / gm + (fx * r1 + fy * r2 + fz * r3) / POW(gm, 3);

        r1 = (fyy * fzz - fyz * fyz) * fx + (fzx * fyz - fxy * fzz) * fy + (fxy * fyz - fzx * fyy) * fz;
        r2 = (fyz * fzx - fxy * fzz) * fx + (fxx * fzz - fzx * fzx) * fy + (fzx * fxy - fxx * fyz) * fz;
        r3 = (fxy * fyz - fyy * fzx) * fx + (fzx * fxy - fxx * fyz) * fy + (fxx * fyy - fxy * fxy) * fz;
        GaussianCurvature[c] = (fx * r1 + fy * r2 + fz * r3) / POW(gm, 4);

        double px = (HPrimal[xp] - HPrimal[xm]) / (2 * dx);
        double py = (HPrimal[yp] - HPrimal[ym]) / (2 * dy);
        double pz = (HPrimal[zp] - HPrimal[zm]) / (2 * dz);
        double dot = px * fx + py * fy + pz * fz;
        Heaviside[c] = dot / POW(gm, 2);

        double pxx = (HPrimal[xp] - 2 * HPrimal[c] + HPrimal[xm]) / (dx * dx);
        double pyy = (HPrimal[yp] - 2 * HPrimal[c] + HPrimal[ym]) / (dy * dy);
        double pzz = (HPrimal[zp] - 2 * HPrimal[c] + HPrimal[zm]) / (dz * dz);
        double plap = pxx + pyy + pzz;
        DiracDelta[c] = plap / POW(gm, 2) - dot * lap / POW(gm, 4);
    }
}

/* ------------------------------------------------------------------------------------ */
/* ENORK2: second-order ENO with the sub-cell fix and Heun RK2 (Min 2010)                */
/*   1_0_ENORK2_Reinitialization/boundary_correction.cu                                  */
/*   2_0_ENORK2_Extend/enork2_extend.cu                                                  */
/* ------------------------------------------------------------------------------------ */

/* line values v4, v1, v0, v2, v3 = f[-2..+2] along an axis */
static inline void line5(const double *f, const grid3 *g, int i, int j, int k, int axis, double v[5])
{
    for (int s = -2; s <= 2; ++s) v[s + 2] = f[step_node(g, i, j, k, axis, s)];
}

/* Second-order ENO one-sided derivatives at v0 with the interface at pr / pl where they
 * differ from ds; the value at the interface is vf / vb (0 for reinitialization).
 * eno_derivative, boundary_correction.cu:81-101; eno_derivative_field,
 * enork2_extend.cu:56-75. */
static void eno2_derivative(const double v[5], double pr, double pl, double ds, double vf, double vb, double *sR,
                            double *sL)
{
    double v4 = v[0], v1 = v[1], v0 = v[2], v2 = v[3], v3 = v[4];
    double p2m;
    double p2 = v1 - 2.0 * v0 + v2;
    double p2r = v0 - 2.0 * v2 + v3;
    p2m = 0.5 * minmod(p2, p2r) / POW(ds, 2);
    double vr = (pr == ds) ? v2 : vf;
    *sR = (vr - v0) / pr - pr * p2m;
    double p2l = v0 - 2.0 * v1 + v4;
    p2m = 0.5 * minmod(p2, p2l) / POW(ds, 2);
    double vl = (pl == ds) ? v1 : vb;
    *sL = (v0 - vl) / pl + pl * p2m;
}

/* boundary_correction (ENORK2), boundary_correction.cu:104-146: quadratic-ENO distance at
 * every crossed edge, scatter form (entries without a crossing keep the caller's value). */
void orc_enork2_boundary_correction(double *xpr, double *xpl, double *ypf, double *ypb, double *zpu, double *zpd,
                                    const double *lsf, int num_ele, int rows, int cols, int pges, double dx,
                                    double dy, double dz)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        double f0 = lsf[c];
        for (int ax = 0; ax < 3; ++ax) {
            int64_t nb = step_node(&g, i, j, k, ax, 1);
            double f2 = lsf[nb];
            if (f0 * f2 < 0) {
                fore[ax][c] = eno2_distance(lsf[step_node(&g, i, j, k, ax, -1)], f0, f2,
                                            lsf[step_node(&g, i, j, k, ax, 2)], h[ax]);
                back[ax][nb] = h[ax] - fore[ax][c];
            }
        }
    }
}

/* re_step (ENORK2), boundary_correction.cu:148-200: Godunov Hamiltonian with the
 * second-order ENO derivatives; no fixed-node test. */
void orc_enork2_re_step(double *step, const double *lsf, const bool *mask, const double *deltat, const double *xpr,
                        const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                        const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                        int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        double df[3], db[3];
        for (int ax = 0; ax < 3; ++ax) {
            double v[5];
            line5(lsf, &g, i, j, k, ax, v);
            eno2_derivative(v, fore[ax][c], back[ax][c], h[ax], 0, 0, &df[ax], &db[ax]);
        }
        double xR = df[0], xL = db[0], yF = df[1], yB = db[1], zU = df[2], zD = db[2];
        if (mask[c]) {
            step[c] = (sqrt(dmax(POW(dmin(0, xL), 2), POW(dmax(0, xR), 2)) + dmax(POW(dmin(0, yB), 2), POW(dmax(0, yF), 2)) +
                            dmax(POW(dmin(0, zD), 2), POW(dmax(0, zU), 2))) - 1) * deltat[c] * (-1.);
        } else {
            step[c] = (sqrt(dmax(POW(dmax(0, xL), 2), POW(dmin(0, xR), 2)) + dmax(POW(dmax(0, yB), 2), POW(dmin(0, yF), 2)) +
                            dmax(POW(dmax(0, zD), 2), POW(dmin(0, zU), 2))) - 1) * deltat[c] * (1.);
        }
    }
}

/* upwind_normal (ENORK2), enork2_extend.cu:82-141: per axis the ENO derivative toward the
 * side whose neighbour value (0 across the interface) is smaller in magnitude. */
void orc_enork2_upwind_normal(double *nx, double *ny, double *nz, const double *lsf, const double *xpr,
                              const double *xpl, const double *ypf, const double *ypb, const double *zpu,
                              const double *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                              int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    double *n[3] = {nx, ny, nz};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        for (int ax = 0; ax < 3; ++ax) {
            double v[5], sR, sL;
            line5(lsf, &g, i, j, k, ax, v);
            double pr = fore[ax][c], pl = back[ax][c];
            eno2_derivative(v, pr, pl, h[ax], 0, 0, &sR, &sL);
            double vr = (pr == h[ax]) ? v[3] : 0;
            double vl = (pl == h[ax]) ? v[1] : 0;
            n[ax][c] = (fabs(vr) < fabs(vl)) ? sR : sL;
        }
    }
}

/* cubic_eno_interp, enork2_extend.cu:144-172: the quadratic ENO interpolant of the cell
 * cut by the interface, evaluated at the crossing (0 where there is none). */
static void eno2_crossing(const double v[5], double dis_f, double dis_b, double ds, double *cf, double *cb)
{
    double v4 = v[0], v1 = v[1], v0 = v[2], v2 = v[3], v3 = v[4];
    *cf = 0;
    *cb = 0;
    if (dis_f != ds) {
        double p2 = v2 - 2.0 * v0 + v1;
        double p2r = v3 - 2.0 * v2 + v0;
        double c2 = 0.5 * minmod(p2, p2r) / POW(ds, 2);
        double c1 = (v2 - v0) / ds;
        double c0 = (v2 + v0) / 2 - c2 * POW(ds, 2) / 4;
        double x = dis_f - ds / 2;
        *cf = c2 * x * x + c1 * x + c0;
    }
    if (dis_b != ds) {
        double p2 = v2 - 2.0 * v0 + v1;
        double p2l = v0 - 2.0 * v1 + v4;
        double c2 = 0.5 * minmod(p2, p2l) / POW(ds, 2);
        double c1 = (v0 - v1) / ds;
        double c0 = (v1 + v0) / 2 - c2 * POW(ds, 2) / 4;
        double x = ds / 2 - dis_b;
        *cb = c2 * x * x + c1 * x + c0;
    }
}

/* boundary_interpolate (ENORK2), enork2_extend.cu:175-211: every entry is written. */
void orc_enork2_boundary_interpolate(double *cpr, double *cpl, double *cpf, double *cpb, double *cpu, double *cpd,
                                     const double *xpr, const double *xpl, const double *ypf, const double *ypb,
                                     const double *zpu, const double *zpd, const double *lsf, int rows, int cols,
                                     int pges, double dx, double dy, double dz, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    double *cf[3] = {cpr, cpf, cpu}, *cb[3] = {cpl, cpb, cpd};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    double h[3] = {dx, dy, dz};
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        for (int ax = 0; ax < 3; ++ax) {
            double v[5];
            line5(lsf, &g, i, j, k, ax, v);
            eno2_crossing(v, fore[ax][c], back[ax][c], h[ax], &cf[ax][c], &cb[ax][c]);
        }
    }
}

/* extend_step (ENORK2), enork2_extend.cu:214-267: upwind transport with the ENO
 * derivatives whose interface values are the crossing values; no fixed-node test. */
void orc_enork2_extend_step(double *step, const double *deltat, const double *lsf, const double *vx,
                            const double *vy, const double *vz, const double *xpr, const double *xpl,
                            const double *ypf, const double *ypb, const double *zpu, const double *zpd,
                            const double *cpr, const double *cpl, const double *cpf, const double *cpb,
                            const double *cpu, const double *cpd, int rows, int cols, int pges, double dx, double dy,
                            double dz, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    const double *v[3] = {vx, vy, vz};
    const double *fore[3] = {xpr, ypf, zpu}, *back[3] = {xpl, ypb, zpd};
    const double *cf[3] = {cpr, cpf, cpu}, *cb[3] = {cpl, cpb, cpd};
    double h[3] = {dx, dy, dz};
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        double df[3], db[3];
        for (int ax = 0; ax < 3; ++ax) {
            double w[5];
            line5(lsf, &g, i, j, k, ax, w);
            eno2_derivative(w, fore[ax][c], back[ax][c], h[ax], cf[ax][c], cb[ax][c], &df[ax], &db[ax]);
        }
        step[c] = (dmin(0, v[0][c]) * df[0] + dmax(0, v[0][c]) * db[0] + dmin(0, v[1][c]) * df[1] +
                   dmax(0, v[1][c]) * db[1] + dmin(0, v[2][c]) * df[2] + dmax(0, v[2][c]) * db[2]) *
                  deltat[c];
    }
}

/* auxi_set_calculus_toolbox (auxi_set_calculus_toolbox.cu:10-199): the toolbox of the
 * auxiliary level set A on the surface of F.  Central differences of A (clamped), the
 * tangent t = (grad F x grad A) / |grad F x grad A| of the curve A = 0 on F = 0, the
 * conormal n = t x N, geodesic and normal curvature, geodesic torsion, the perpendicular
 * curvature, and the Heaviside/Dirac functions of A from the primal AHPrimal = max(A, 0);
 * F's toolbox fields are inputs.  Vector norms are floored at 1e-14 (norm(),
 * shared_utilities.cup:8-12). */
static inline double norm3(double x, double y, double z) { return dmax(sqrt(x * x + y * y + z * z), 1e-14); }

void orc_auxi_set_calculus_toolbox(
    double *Ax, double *Ay, double *Az, double *AGradMag, double *ACx, double *ACy, double *ACz,
    double *ANormCrossAF, double *Tx, double *Ty, double *Tz, double *Anx, double *Any, double *Anz, double *Axx,
    double *Ayy, double *Azz, double *Axy, double *Ayz, double *Azx, double *ALaplacian, double *GeodesicCurvature,
    double *NormalCurvature, double *GeodesicTorsion, double *BPerpendicular, double *AHeaviside,
    double *ADiracDelta, const double *lsf, const double *AHPrimal, const double *Fx, const double *Fy,
    const double *Fz, const double *FGradMag, const double *Nx, const double *Ny, const double *Nz,
    const double *Fxx, const double *Fyy, const double *Fzz, const double *Fxy, const double *Fyz,
    const double *Fzx, int rows, int cols, int pges, double dx, double dy, double dz, double ds, int num_ele)
{
    (void)num_ele;
    grid3 g = {rows, cols, pges};
    FOR_EACH_NODE(g)
    {
        int64_t c = node(&g, i, j, k);
        int64_t xp = node(&g, i, j + 1, k), xm = node(&g, i, j - 1, k);
        int64_t yp = node(&g, i + 1, j, k), ym = node(&g, i - 1, j, k);
        int64_t zp = node(&g, i, j, k + 1), zm = node(&g, i, j, k - 1);
        const double *a = lsf;
        double ax = (a[xp] - a[xm]) / (2 * dx);
        double ay = (a[yp] - a[ym]) / (2 * dy);
        double az = (a[zp] - a[zm]) / (2 * dz);
        double agm = norm3(ax, ay, az);
        Ax[c] = ax;
        Ay[c] = ay;
        Az[c] = az;
        AGradMag[c] = agm;

        double fx = Fx[c], fy = Fy[c], fz = Fz[c];
        double cx = fy * az - fz * ay, cy = fz * ax - fx * az, cz = fx * ay - fy * ax;
        double ncr = norm3(cx, cy, cz);
        ACx[c] = cx;
        ACy[c] = cy;
        ACz[c] = cz;
        ANormCrossAF[c] = ncr;
        double tx = cx / ncr, ty = cy / ncr, tz = cz / ncr;
        Tx[c] = tx;
        Ty[c] = ty;
        Tz[c] = tz;
        double fnx = Nx[c], fny = Ny[c], fnz = Nz[c];
        double nx = ty * fnz - tz * fny, ny = tz * fnx - tx * fnz, nz = tx * fny - ty * fnx;
        Anx[c] = nx;
        Any[c] = ny;
        Anz[c] = nz;

        double axx = (a[xp] - 2 * a[c] + a[xm]) / (dx * dx);
        double ayy = (a[yp] - 2 * a[c] + a[ym]) / (dy * dy);
        double azz = (a[zp] - 2 * a[c] + a[zm]) / (dz * dz);
        double axy = (a[node(&g, i + 1, j + 1, k)] + a[node(&g, i - 1, j - 1, k)] - a[node(&g, i + 1, j - 1, k)] -
                      a[node(&g, i - 1, j + 1, k)]) / (4 * ds * ds);
        double ayz = (a[node(&g, i + 1, j, k + 1)] + a[node(&g, i - 1, j, k - 1)] - a[node(&g, i + 1, j, k - 1)] -
                      a[node(&g, i - 1, j, k + 1)]) / (4 * ds * ds);
        double azx = (a[node(&g, i, j + 1, k + 1)] + a[node(&g, i, j - 1, k - 1)] - a[node(&g, i, j + 1, k - 1)] -
                      a[node(&g, i, j - 1, k + 1)]) / (4 * ds * ds);
        double alap = axx + ayy + azz;
        Axx[c] = axx;
        Ayy[c] = ayy;
        Azz[c] = azz;
        Axy[c] = axy;
        Ayz[c] = ayz;
        Azx[c] = azx;
        ALaplacian[c] = alap;

        double fxx = Fxx[c], fyy = Fyy[c], fzz = Fzz[c], fxy = Fxy[c], fyz = Fyz[c], fzx = Fzx[c];
        double fgm = FGradMag[c];
        /* geodesic curvature: n . ((H_F t) x grad A + grad F x (H_A t)) / |grad F x grad A| */
        double vx = tx * fxx + ty * fxy + tz * fzx;
        double vy = tx * fxy + ty * fyy + tz * fyz;
        double vz = tx * fzx + ty * fyz + tz * fzz;
        double w1x = vy * az - vz * ay, w1y = vz * ax - vx * az, w1z = vx * ay - vy * ax;
        vx = tx * axx + ty * axy + tz * azx;
        vy = tx * axy + ty * ayy + tz * ayz;
        vz = tx * azx + ty * ayz + tz * azz;
        double w2x = fy * vz - fz * vy, w2y = fz * vx - fx * vz, w2z = fx * vy - fy * vx;
        GeodesicCurvature[c] = (nx * (w1x + w2x) + ny * (w1y + w2y) + nz * (w1z + w2z)) / ncr;

        /* grad N = H_F / |grad F| - grad F (H_F grad F)^T / |grad F|^3, row by row */
        double g3 = POW(fgm, 3);
        double Nxx = fxx / fgm - fx * (fxx * fx + fxy * fy + fzx * fz) / g3;
        double Nyx = fxy / fgm - fy * (fxx * fx + fxy * fy + fzx * fz) / g3;
        double Nzx = fzx / fgm - fz * (fxx * fx + fxy * fy + fzx * fz) / g3;
        double Nxy = fxy / fgm - fx * (fxy * fx + fyy * fy + fyz * fz) / g3;
        double Nyy = fyy / fgm - fy * (fxy * fx + fyy * fy + fyz * fz) / g3;
        double Nzy = fyz / fgm - fz * (fxy * fx + fyy * fy + fyz * fz) / g3;
        double Nxz = fzx / fgm - fx * (fzx * fx + fyz * fy + fzz * fz) / g3;
        double Nyz = fyz / fgm - fy * (fzx * fx + fyz * fy + fzz * fz) / g3;
        double Nzz = fzz / fgm - fz * (fzx * fx + fyz * fy + fzz * fz) / g3;
        vx = Nxx * tx + Nxy * ty + Nxz * tz;
        vy = Nyx * tx + Nyy * ty + Nyz * tz;
        vz = Nzx * tx + Nzy * ty + Nzz * tz;
        NormalCurvature[c] = -(tx * vx + ty * vy + tz * vz);
        vx = Nxx * nx + Nxy * ny + Nxz * nz;
        vy = Nyx * nx + Nyy * ny + Nyz * nz;
        vz = Nzx * nx + Nzy * ny + Nzz * nz;
        GeodesicTorsion[c] = -(tx * vx + ty * vy + tz * vz);
        BPerpendicular[c] = -(nx * vx + ny * vy + nz * vz);

        const double *p = AHPrimal;
        double px = (p[xp] - p[xm]) / (2 * dx);
        double py = (p[yp] - p[ym]) / (2 * dy);
        double pz = (p[zp] - p[zm]) / (2 * dz);
        double dot = px * ax + py * ay + pz * az;
        AHeaviside[c] = dot / POW(agm, 2);
        double pxx = (p[xp] - 2 * p[c] + p[xm]) / (dx * dx);
        double pyy = (p[yp] - 2 * p[c] + p[ym]) / (dy * dy);
        double pzz = (p[zp] - 2 * p[c] + p[zm]) / (dz * dz);
        double plap = pxx + pyy + pzz;
        ADiracDelta[c] = plap / POW(agm, 2) - dot * alap / POW(agm, 4);
    }
}

int orc_version(void) { return 1; }
