// vsl_device.cuh -- device building blocks of the level-set hot path (sm_103a).
//
// Grid layout (the reference's MATLAB layout): ind = k*rows*cols + j*rows + i, with
// i = row (y, stride 1), j = column (x, stride rows), k = page (z, stride rows*cols).
// Neighbour coordinates outside the grid are clamped to the edge, as the reference's
// sub2ind does (CUDA_Code/1_3_WENO5RK3_Reinitialization/shared_utilities.hpp:21-31).
//
// Stencil arithmetic is templated on the field type T (double for the plain form, float
// for the mixed-precision form).  The sub-cell interface distances (polynomial fits and
// their roots) are always computed in double.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vsl {

// ---------------------------------------------------------------------------------------
// grid and indexing
// ---------------------------------------------------------------------------------------

struct Grid {
    int rows, cols, pges;
    long long plane;  // rows * cols
    long long num;    // rows * cols * pges
    double dx, dy, dz;
};

__host__ __device__ inline Grid make_grid(int rows, int cols, int pges, double dx, double dy, double dz)
{
    Grid g;
    g.rows = rows;
    g.cols = cols;
    g.pges = pges;
    g.plane = (long long)rows * cols;
    g.num = g.plane * pges;
    g.dx = dx;
    g.dy = dy;
    g.dz = dz;
    return g;
}

enum Axis { AX_X = 0, AX_Y = 1, AX_Z = 2 };

__device__ __forceinline__ int clampi(int v, int n) { return min(max(v, 0), n - 1); }

__device__ __forceinline__ long long node_index(const Grid &g, int i, int j, int k)
{
    return (long long)k * g.plane + (long long)j * g.rows + i;
}

__device__ __forceinline__ long long clamped_index(const Grid &g, int i, int j, int k)
{
    return node_index(g, clampi(i, g.rows), clampi(j, g.cols), clampi(k, g.pges));
}

// Coordinate, extent and stride of (i,j,k) along an axis; `base` is the index with that
// coordinate set to zero.
struct AxisLine {
    long long base;
    long long stride;
    int c, n;
};

__device__ __forceinline__ AxisLine axis_line(const Grid &g, int i, int j, int k, int ax)
{
    AxisLine L;
    if (ax == AX_X) {
        L.base = (long long)k * g.plane + i;
        L.stride = g.rows;
        L.c = j;
        L.n = g.cols;
    } else if (ax == AX_Y) {
        L.base = (long long)k * g.plane + (long long)j * g.rows;
        L.stride = 1;
        L.c = i;
        L.n = g.rows;
    } else {
        L.base = (long long)j * g.rows + i;
        L.stride = g.plane;
        L.c = k;
        L.n = g.pges;
    }
    return L;
}

// Seven values f[c-3 .. c+3] along a line, clamped.
template <typename T>
__device__ __forceinline__ void load_line7(const T *__restrict__ f, const AxisLine &L, T p[7])
{
#pragma unroll
    for (int s = -3; s <= 3; ++s) p[s + 3] = __ldg(f + L.base + (long long)clampi(L.c + s, L.n) * L.stride);
}

__device__ __forceinline__ double axis_h(const Grid &g, int ax) { return ax == AX_X ? g.dx : (ax == AX_Y ? g.dy : g.dz); }

// ---------------------------------------------------------------------------------------
// scalar helpers (shared_utilities.hpp:5-18): comparisons written as in the reference so
// ties and signed zeros resolve the same way.
// ---------------------------------------------------------------------------------------

template <typename T> __device__ __forceinline__ T vmax(T x, T y) { return (x < y) ? y : x; }
template <typename T> __device__ __forceinline__ T vmin(T x, T y) { return (x < y) ? x : y; }
template <typename T> __device__ __forceinline__ T minmod(T x, T y)
{
    return (x * y < T(0)) ? T(0) : (fabs(x) < fabs(y) ? x : y);
}
template <typename T> __device__ __forceinline__ T minabs(T x, T y) { return (fabs(x) < fabs(y)) ? x : y; }
__device__ __forceinline__ double sgn1(double x) { return (x > 0) ? 1.0 : -1.0; }
template <typename T> __device__ __forceinline__ T sqr(T x) { return x * x; }

// t^p rounded once: the running product is carried as an unevaluated double-double
// (hi + lo, error-free products via fma), so the result is the correctly rounded power
// except in cases within ~2^-100 of a rounding midpoint -- what a correctly rounded
// pow(t, p) returns.  The reference's polynomial and curvature code calls pow(t, p).
template <int P> __device__ __forceinline__ double pow_cr(double t)
{
    if (P == 0) return 1.0;
    if (P == 1) return t;
    double hi = t, lo = 0.0;
#pragma unroll
    for (int k = 2; k <= P; ++k) {
        const double p1 = hi * t;
        const double e1 = fma(hi, t, -p1);
        lo = fma(lo, t, e1);
        hi = p1;
    }
    return hi + lo;
}

// ---------------------------------------------------------------------------------------
// sub-cell interface distances, always double
// ---------------------------------------------------------------------------------------

// Degree-n interpolant through (x[m], y[m]) in monomial form: expand each Lagrange basis
// term factor by factor (highest power first) and sum per power.  Same construction as
// Poly<n>::setInterpolation (shared_utilities.hpp:55-103).
template <int N>
__device__ __forceinline__ void lagrange_monomial(const double *x, const double *y, double *a)
{
    double scale[N + 1], ex[N + 1][N + 1];
#pragma unroll
    for (int m = 0; m <= N; ++m) {
        scale[m] = y[m];
        ex[m][0] = 1.0;
#pragma unroll
        for (int q = 1; q <= N; ++q) ex[m][q] = 0.0;
        int r = 0;
#pragma unroll
        for (int q = 0; q <= N; ++q) {
            if (q == m) continue;
            scale[m] /= x[m] - x[q];
            // multiply the running product by (t - x[q])
#pragma unroll
            for (int p = N; p >= 1; --p)
                if (p <= r + 1) ex[m][p] = ex[m][p] - x[q] * ex[m][p - 1];
            ++r;
        }
    }
#pragma unroll
    for (int p = 0; p <= N; ++p) {
        double acc = 0.0;
#pragma unroll
        for (int m = 0; m <= N; ++m) acc += scale[m] * ex[m][N - p];
        a[p] = acc;
    }
}

// sum of a[p] t^p, terms added from p = 0 (Poly<n>::operator(), shared_utilities.hpp:47-53)
template <int N> __device__ __forceinline__ double poly_eval(const double *a, double t)
{
    double v = 0.0;
    v += a[0] * 1.0;
    if (N >= 1) v += a[1] * t;
    if (N >= 2) v += a[2] * (t * t);
    if (N >= 3) v += a[3] * pow_cr<3>(t);
    if (N >= 4) v += a[4] * pow_cr<4>(t);
    if (N >= 5) v += a[5] * pow_cr<5>(t);
    return v;
}

// Brent's root finder over [x1, x2] (tolerance tol, at most 100 iterations), the method
// of zeroin (shared_utilities.hpp:109-173).
template <int N> __device__ double brent_root(const double *a, double x1, double x2, double tol)
{
    double d = 0.0, e = 0.0;
    double lo = x1, b = x2, c = x2;
    double flo = poly_eval<N>(a, lo), fb = poly_eval<N>(a, b), fc = fb;
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
        double xm = 0.5 * (c - b);
        if (fabs(xm) <= tol || fb == 0.0) return b;
        if (fabs(e) < tol || fabs(flo) <= fabs(fb)) {
            d = xm;
            e = xm;
        } else {
            double s = fb / flo, p, q;
            if (lo == c) {
                p = 2.0 * xm * s;
                q = 1.0 - s;
            } else {
                double qq = flo / fc, r = fb / fc;
                p = s * (2.0 * xm * qq * (qq - r) - (b - lo) * (r - 1.0));
                q = (qq - 1.0) * (r - 1.0) * (s - 1.0);
            }
            if (p > 0) q = -q;
            p = fabs(p);
            double lim1 = 3.0 * xm * q - fabs(tol * q);
            double lim2 = fabs(e * q);
            if (2.0 * p < vmin(lim1, lim2)) {
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
            b += sgn1(xm) * tol;
        fb = poly_eval<N>(a, b);
    }
    return b;
}

// Quadratic ENO distance from node b to the interface between b and c; a before b, d
// after c (sp, boundary_location.cu:6-20).
__device__ __forceinline__ double eno2_distance(double a, double b, double c, double d, double h)
{
    const double eps = 10e-10;
    double d2 = minmod(c - 2.0 * b + a, d - 2.0 * c + b);
    if (d2 > eps || d2 < -eps) {
        double disc = sqr(0.5 * d2 - b - c) - 4. * b * c;
        return h * (0.5 + (b - c - sgn1(b - c) * sqrt(disc)) / d2);
    }
    return h * b / (b - c);
}

// Degree-5 fit through samples at 0..5h with the crossing between 2h and 3h; quadratic
// ENO next to a kink (six_distance, boundary_location.cu:53-80).
__device__ inline double quintic_distance(const double v[6], double h)
{
    if (v[1] * v[2] < 0 || v[3] * v[4] < 0) return eno2_distance(v[1], v[2], v[3], v[4], h);
    double xs[6] = {0.0, h, 2 * h, 3 * h, 4 * h, 5 * h};
    double a[6];
    lagrange_monomial<5>(xs, v, a);
    double t = brent_root<5>(a, 2 * h, 3 * h, 3e-16);
    t = vmin(vmax(t, 2 * h), 3 * h);
    return t - 2 * h;
}

// Cubic through 0..3h, Newton from the linear guess, at most 50 steps (cubic_distance,
// weno_rk3_reinitialization.cu:73-116).
__device__ inline double cubic_newton_distance(double v0, double v1, double v2, double v3, double h)
{
    if (v0 * v1 < 0 || v2 * v3 < 0) return eno2_distance(v0, v1, v2, v3, h);
    double a0 = v0;
    double a1 = (3.0 * (v1 - v0) - 3.0 / 2.0 * (v2 - v0) + 1.0 / 3.0 * (v3 - v0)) / h;
    double a2 = (-5.0 / 2.0 * (v1 - v0) + 2.0 * (v2 - v0) - 1.0 / 2.0 * (v3 - v0)) / (h * h);
    double a3 = (1.0 / 2.0 * (v1 - v0) - 1.0 / 2.0 * (v2 - v0) + 1.0 / 6.0 * (v3 - v0)) / pow_cr<3>(h);
    double t = h + h * v1 / (v1 - v2);
    double change = 1.0;
    for (int it = 0; change > 1e-14 && it < 50; ++it) {
        double f = a0 + a1 * t + a2 * t * t + a3 * t * t * t;
        double df = a1 + 2 * a2 * t + 3 * a3 * t * t;
        double r = f / df;
        change = fabs(r);
        t = t - r;
    }
    t = vmin(vmax(t, h), 2 * h);
    return t - h;
}

// Distance from the node at L.c to the interface between it and its +1 neighbour along
// the line L, as the reference thread of that node computes it (double arithmetic on
// the promoted samples): degree-5 fit (boundary_location.cu:84-132) or cubic Newton
// (weno_rk3_reinitialization.cu:251-293).
template <bool QUINTIC, typename T>
__device__ __forceinline__ double fore_distance(const T *__restrict__ f, const AxisLine &L, double h)
{
    if (QUINTIC) {
        double v[6];
#pragma unroll
        for (int s = -2; s <= 3; ++s) v[s + 2] = (double)__ldg(f + L.base + (long long)clampi(L.c + s, L.n) * L.stride);
        return quintic_distance(v, h);
    } else {
        double v0 = (double)__ldg(f + L.base + (long long)clampi(L.c - 1, L.n) * L.stride);
        double v1 = (double)__ldg(f + L.base + (long long)L.c * L.stride);
        double v2 = (double)__ldg(f + L.base + (long long)clampi(L.c + 1, L.n) * L.stride);
        double v3 = (double)__ldg(f + L.base + (long long)clampi(L.c + 2, L.n) * L.stride);
        return cubic_newton_distance(v0, v1, v2, v3, h);
    }
}

// ---------------------------------------------------------------------------------------
// one-sided derivatives
// ---------------------------------------------------------------------------------------

// Jiang-Shu WENO5 one-sided derivative from five first differences (biased toward v3),
// in the reference's operation order (re_step.cu:11-37); squares by multiplication.
template <typename T>
__device__ __forceinline__ T weno5_plain(T v1, T v2, T v3, T v4, T v5)
{
    T q1 = T(1. / 3.) * v1 - T(7. / 6.) * v2 + T(11. / 6.) * v3;
    T q2 = T(-1. / 6.) * v2 + T(5. / 6.) * v3 + T(1. / 3.) * v4;
    T q3 = T(1. / 3.) * v3 + T(5. / 6.) * v4 - T(1. / 6.) * v5;
    T s1 = T(13. / 12.) * sqr(v1 - 2 * v2 + v3) + T(1. / 4.) * sqr(v1 - 4 * v2 + 3 * v3);
    T s2 = T(13. / 12.) * sqr(v2 - 2 * v3 + v4) + T(1. / 4.) * sqr(v2 - v4);
    T s3 = T(13. / 12.) * sqr(v3 - 2 * v4 + v5) + T(1. / 4.) * sqr(3 * v3 - 4 * v4 + v5);
    const T eps = T(1e-6);
    T a1 = T(0.1) / sqr(s1 + eps);
    T a2 = T(0.6) / sqr(s2 + eps);
    T a3 = T(0.3) / sqr(s3 + eps);
    T tot = a1 + a2 + a3;
    return (a1 / tot) * q1 + (a2 / tot) * q2 + (a3 / tot) * q3;
}

// a / b: the hardware reciprocal-based quotient for float (about 2 ulp), IEEE for double
// The hardware approximate reciprocal (PTX rcp.approx.ftz.f32).  The WENO5 weights and
// quotients divide by (S + eps)^2 and by sums of such weights: normal numbers far inside the
// FP32 range for any grid spacing above ~1e-6, where a * rcp_ftz(b) is the value
// __fdividef(a, b) returns (checked bitwise on the GPU against the __fdividef form) without
// the subnormal and range handling a general quotient carries.
__device__ __forceinline__ float rcp_ftz(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float fast_div(float a, float b) { return a * rcp_ftz(b); }
__device__ __forceinline__ double fast_div(double a, double b) { return a / b; }

// The same reconstruction from UNSCALED differences u = h*v with eps2 = eps*h^2 and the
// 1/h factor applied once at the end (S_k(u) = h^2 S_k(v), so the normalised weights are
// unchanged); the weights use the fast quotient.  Algebraically identical to
// weno5_plain(u/h) * h; used by the mixed-precision form only.
template <typename T>
__device__ __forceinline__ T weno5_fast(T u1, T u2, T u3, T u4, T u5, T eps2)
{
    T q1 = T(1. / 3.) * u1 - T(7. / 6.) * u2 + T(11. / 6.) * u3;
    T q2 = T(-1. / 6.) * u2 + T(5. / 6.) * u3 + T(1. / 3.) * u4;
    T q3 = T(1. / 3.) * u3 + T(5. / 6.) * u4 - T(1. / 6.) * u5;
    T s1 = T(13. / 12.) * sqr(u1 - 2 * u2 + u3) + T(1. / 4.) * sqr(u1 - 4 * u2 + 3 * u3);
    T s2 = T(13. / 12.) * sqr(u2 - 2 * u3 + u4) + T(1. / 4.) * sqr(u2 - u4);
    T s3 = T(13. / 12.) * sqr(u3 - 2 * u4 + u5) + T(1. / 4.) * sqr(3 * u3 - 4 * u4 + u5);
    T a1 = fast_div(T(0.1), sqr(s1 + eps2));
    T a2 = fast_div(T(0.6), sqr(s2 + eps2));
    T a3 = fast_div(T(0.3), sqr(s3 + eps2));
    return fast_div(a1 * q1 + a2 * q2 + a3 * q3, a1 + a2 + a3);
}

// Smoothness indicators of the three candidate stencils of a WENO5 window of five first
// differences (unscaled), returned as the reciprocal squares 1/(S_k + eps2)^2.  A window
// serves two derivatives: the backward one at its fourth node and, reversed, the forward
// one at its third node, since S_1(a,b,c) = S_3(c,b,a) and S_2 is symmetric.
__device__ __forceinline__ void weno5_window_weights(float u1, float u2, float u3, float u4, float u5, float eps2,
                                                     float &r1, float &r2, float &r3)
{
    const float s1 = (13.f / 12.f) * sqr(u1 - 2 * u2 + u3) + 0.25f * sqr(u1 - 4 * u2 + 3 * u3);
    const float s2 = (13.f / 12.f) * sqr(u2 - 2 * u3 + u4) + 0.25f * sqr(u2 - u4);
    const float s3 = (13.f / 12.f) * sqr(u3 - 2 * u4 + u5) + 0.25f * sqr(3 * u3 - 4 * u4 + u5);
    r1 = rcp_ftz(sqr(s1 + eps2));
    r2 = rcp_ftz(sqr(s2 + eps2));
    r3 = rcp_ftz(sqr(s3 + eps2));
}

// WENO5 one-sided derivative (unscaled differences, biased toward u3) with the reciprocal
// weights of its window given: weno5_fast with the smoothness part precomputed.
__device__ __forceinline__ float weno5_with_weights(float u1, float u2, float u3, float u4, float u5, float r1,
                                                    float r2, float r3)
{
    const float q1 = (1.f / 3.f) * u1 - (7.f / 6.f) * u2 + (11.f / 6.f) * u3;
    const float q2 = (-1.f / 6.f) * u2 + (5.f / 6.f) * u3 + (1.f / 3.f) * u4;
    const float q3 = (1.f / 3.f) * u3 + (5.f / 6.f) * u4 - (1.f / 6.f) * u5;
    const float a1 = 0.1f * r1, a2 = 0.6f * r2, a3 = 0.3f * r3;
    return (a1 * q1 + a2 * q2 + a3 * q3) * rcp_ftz(a1 + a2 + a3);
}

// Seven-point stencil with the interface inserted at r1 (forward) / l1 (backward) when
// they are shorter than h, carrying the values hf / hb there (select_stencil,
// re_step.cu:41-77 and shared_utilities.cup:211-247).
template <typename T>
__device__ __forceinline__ void insert_interface(const T p[7], T r1, T l1, T h, T hf, T hb, T xs[7], T hs[7])
{
    hs[3] = p[3];
    xs[3] = T(0);
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

// Smoothness indicators of the nonuniform WENO reconstruction for faces e[0..5] and
// cell averages u[0..4] (re_step.cu:116-158; the same expressions serve both biases).
template <typename T>
__device__ __forceinline__ void nu_smoothness(const T e[6], const T u[5], T s[3])
{
    const T xm25 = e[0], xm15 = e[1], xm05 = e[2], x05 = e[3], x15 = e[4], x25 = e[5];
    const T um2 = u[0], um1 = u[1], u0 = u[2], u1 = u[3], u2 = u[4];
    const T w = x05 - xm05;
    s[0] = T(4.0) * sqr(w / (x25 - xm05)) *
           (sqr((u2 - u1) / (x25 - x05)) * (T(10.0) * sqr(w) + (x15 - xm05) * (x15 - x05)) +
            (u2 - u1) * (u0 - u1) / ((x25 - x05) * (x15 - xm05)) *
                (T(20.0) * sqr(w) + T(2.0) * (x15 - xm05) * (x15 - x05) + (x25 - xm05) * (T(2.0) * x15 - x05 - xm05)) +
            sqr((u0 - u1) / (x15 - xm05)) * (T(10.0) * sqr(w) + (x25 + x15 - T(2.0) * xm05) * (x25 + x15 - x05 - xm05)));
    s[1] = T(4.0) * sqr(w / (x15 - xm15)) *
           (sqr((um1 - u0) / (x05 - xm15)) * (T(10.0) * sqr(w) + (x15 - xm05) * (x15 - x05)) +
            (u1 - u0) * (um1 - u0) / ((x15 - xm05) * (x05 - xm15)) *
                (T(20.0) * sqr(w) - (x15 - x05) * (xm05 - xm15) - (x15 - xm05) * (x05 - xm15)) +
            sqr((u1 - u0) / (x15 - xm05)) * (T(10.0) * sqr(w) + (xm05 - xm15) * (x05 - xm15)));
    s[2] = T(4.0) * sqr(w / (x05 - xm25)) *
           (sqr((um2 - um1) / (xm05 - xm25)) * (T(10.0) * sqr(w) + (x05 - xm15) * (xm05 - xm15)) +
            (u0 - um1) * (um2 - um1) / ((x05 - xm15) * (xm05 - xm25)) *
                (T(20.0) * sqr(w) + T(2.0) * (x05 - xm15) * (xm05 - xm15) + (x05 - xm25) * (x05 + xm05 - T(2.0) * xm15)) +
            sqr((u0 - um1) / (x05 - xm15)) * (T(10.0) * sqr(w) + (T(2.0) * x05 - xm25 - xm15) * (x05 + xm05 - xm15 - xm25)));
}

template <typename T> __device__ __forceinline__ T nu_combine(const T v[3], const T c[3], const T s[3])
{
    const T eps = T(1e-6);
    T a0 = c[0] / sqr(s[0] + eps);
    T a1 = c[1] / sqr(s[1] + eps);
    T a2 = c[2] / sqr(s[2] + eps);
    T tot = a0 + a1 + a2;
    return v[0] * (a0 / tot) + v[1] * (a1 / tot) + v[2] * (a2 / tot);
}

// Nonuniform WENO forward/backward derivatives at xs[3] = 0 (weno_nonuniform,
// re_step.cu:79-243).
template <typename T>
__device__ __noinline__ void weno_nonuniform_pair(const T xs[7], const T hs[7], T &d_fore, T &d_back)
{
    T dd[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) dd[m] = (hs[m + 1] - hs[m]) / (xs[m + 1] - xs[m]);
    T e[6], u[5], v[3], c[3], s[3];
    // forward bias: faces xs[1..6], cells dd[1..5], value at the face xs[3]
#pragma unroll
    for (int m = 0; m < 6; ++m) e[m] = xs[m + 1];
#pragma unroll
    for (int m = 0; m < 5; ++m) u[m] = dd[m + 1];
    {
        const T xm25 = e[0], xm15 = e[1], xm05 = e[2], x05 = e[3], x15 = e[4], x25 = e[5];
        const T um2 = u[0], um1 = u[1], u0 = u[2], u1 = u[3], u2 = u[4];
        v[0] = u1 + (u0 - u1) * (T(1.0) + (x05 - xm05) / (x15 - xm05) + (x05 - xm05) / (x25 - xm05)) +
               (u2 - u1) * ((x05 - xm05) / (x25 - xm05)) * ((x15 - xm05) / (x25 - x05));
        v[1] = u0 + (um1 - u0) * ((x05 - xm05) / (x15 - xm15)) * ((x15 - xm05) / (x05 - xm15)) -
               (u1 - u0) * ((x05 - xm05) / (x15 - xm15)) * ((xm05 - xm15) / (x15 - xm05));
        v[2] = um1 + (u0 - um1) * ((xm05 - xm15) / (x05 - xm25)) * ((xm05 - xm25) / (x05 - xm15)) -
               (um2 - um1) * ((xm05 - xm15) / (x05 - xm25)) * ((x05 - xm05) / (xm05 - xm25));
        c[0] = ((xm05 - xm15) / (x25 - xm25)) * ((xm05 - xm25) / (x25 - xm15));
        c[1] = ((xm05 - xm25) / (x25 - xm25)) * ((x25 - xm05) / (x25 - xm15)) * (T(1.0) + (x25 - xm15) / (x15 - xm25));
        c[2] = ((x15 - xm05) / (x25 - xm25)) * ((x25 - xm05) / (x15 - xm25));
    }
    nu_smoothness(e, u, s);
    d_fore = nu_combine(v, c, s);
    // backward bias: faces xs[0..5], cells dd[0..4], value at the face xs[3]
#pragma unroll
    for (int m = 0; m < 6; ++m) e[m] = xs[m];
#pragma unroll
    for (int m = 0; m < 5; ++m) u[m] = dd[m];
    {
        const T xm25 = e[0], xm15 = e[1], xm05 = e[2], x05 = e[3], x15 = e[4], x25 = e[5];
        const T um2 = u[0], um1 = u[1], u0 = u[2], u1 = u[3], u2 = u[4];
        v[0] = u1 + (u0 - u1) * ((x15 - x05) / (x25 - xm05)) * ((x25 - x05) / (x15 - xm05)) -
               (u2 - u1) * ((x15 - x05) / (x25 - xm05)) * ((x05 - xm05) / (x25 - x05));
        v[1] = u0 + (u1 - u0) * ((x05 - xm05) / (x15 - xm15)) * ((x05 - xm15) / (x15 - xm05)) -
               (um1 - u0) * ((x05 - xm05) / (x15 - xm15)) * ((x15 - x05) / (x05 - xm15));
        v[2] = um1 + (um2 - um1) * ((x05 - xm05) / (xm05 - xm25)) * ((x05 - xm15) / (x05 - xm25)) +
               (u0 - um1) * (T(1.0) + (x05 - xm05) / (x05 - xm15) + (x05 - xm05) / (x05 - xm25));
        c[0] = ((x05 - xm25) / (x25 - xm25)) * ((x05 - xm15) / (x25 - xm15));
        c[1] = ((x05 - xm25) / (x25 - xm25)) * ((x25 - x05) / (x25 - xm15)) * (T(1.0) + (x25 - xm15) / (x15 - xm25));
        c[2] = ((x15 - x05) / (x25 - xm25)) * ((x25 - x05) / (x15 - xm25));
    }
    nu_smoothness(e, u, s);
    d_back = nu_combine(v, c, s);
}

// Nonuniform cubic ENO forward/backward derivatives at xs[3] = 0, the "ENO3" scheme
// (ENO_cubic_derivative, weno_rk3_reinitialization.cu:189-222).
template <typename T>
__device__ __noinline__ void eno3_nonuniform_pair(const T xs[7], const T hs[7], T &d_fore, T &d_back)
{
    const T x3m = xs[0], x2m = xs[1], x1m = xs[2], x0 = xs[3], x1 = xs[4], x2 = xs[5], x3 = xs[6];
    T f25 = (hs[6] - hs[5]) / (x3 - x2);
    T f15 = (hs[5] - hs[4]) / (x2 - x1);
    T f05 = (hs[4] - hs[3]) / (x1 - x0);
    T fm05 = (hs[3] - hs[2]) / (x0 - x1m);
    T fm15 = (hs[2] - hs[1]) / (x1m - x2m);
    T fm25 = (hs[1] - hs[0]) / (x2m - x3m);
    T g2 = (f25 - f15) / (x3 - x1);
    T g1 = (f15 - f05) / (x2 - x0);
    T g0 = (f05 - fm05) / (x1 - x1m);
    T gm1 = (fm05 - fm15) / (x0 - x2m);
    T gm2 = (fm15 - fm25) / (x1m - x3m);
    T t15 = (g2 - g1) / (x3 - x0);
    T t05 = (g1 - g0) / (x2 - x1m);
    T tm05 = (g0 - gm1) / (x1 - x2m);
    T tm15 = (gm1 - gm2) / (x0 - x3m);
    T a1 = (x0 - x1m) * (x0 - x2m) * minabs(tm05, tm15);
    T a2 = (x0 - x1m) * (x0 - x1) * minabs(tm05, t05);
    T a = (fabs(gm1) < fabs(g0)) ? a1 : a2;
    T b1 = (x0 - x1m) * (x0 - x1) * minabs(tm05, t05);
    T b2 = (x0 - x1) * (x0 - x2) * minabs(t05, t15);
    T b = (fabs(g0) < fabs(g1)) ? b1 : b2;
    d_back = fm05 + minmod(gm1, g0) * (x0 - x1m) + a;
    d_fore = f05 + minmod(g0, g1) * (x0 - x1) + b;
}

// Uniform WENO5 pair from the seven line values, plain (reference) numerics.
template <typename T>
__device__ __forceinline__ void weno5_pair_plain(const T p[7], T h, T &d_fore, T &d_back)
{
    T v[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) v[m] = (p[m + 1] - p[m]) / h;
    d_back = weno5_plain(v[0], v[1], v[2], v[3], v[4]);
    d_fore = weno5_plain(v[5], v[4], v[3], v[2], v[1]);
}

// Uniform WENO5 pair, fast numerics (unscaled differences, one division each).
template <typename T>
__device__ __forceinline__ void weno5_pair_fast(const T p[7], T inv_h, T eps2, T &d_fore, T &d_back)
{
    T u[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) u[m] = p[m + 1] - p[m];
    d_back = weno5_fast(u[0], u[1], u[2], u[3], u[4], eps2) * inv_h;
    d_fore = weno5_fast(u[5], u[4], u[3], u[2], u[1], eps2) * inv_h;
}

// Interface-aware pair: nonuniform WENO (eno3 = false) or cubic ENO (eno3 = true).
template <typename T>
__device__ __forceinline__ void interface_pair(const T p[7], T r1, T l1, T h, T hf, T hb, bool eno3, T &d_fore,
                                               T &d_back)
{
    T xs[7], hs[7];
    insert_interface(p, r1, l1, h, hf, hb, xs, hs);
    if (eno3)
        eno3_nonuniform_pair(xs, hs, d_fore, d_back);
    else
        weno_nonuniform_pair(xs, hs, d_fore, d_back);
}

// ---------------------------------------------------------------------------------------
// The interface-aware pair of the mixed (FP32) form, written on the gaps between the seven
// stencil points rather than on their positions.
//
// With the interface at r1 close to h, the position form takes the short gap between the
// interface and the next node as h - r1 in FP32, where r1 is the FP32 rounding of the FP64
// root: a gap of 4e-5 h keeps only about three significant digits, and the one-sided
// divided difference across it (and the WENO weights built on it) inherit that error -- a
// 1e-3 dx error in one pseudo-step at such nodes of a 256^3 grid.  The neighbour beyond the
// crossing stores that same gap as its own distance (h - dist, rounded once from the FP64
// root), so the gap form takes it from there: rc = h - r1 and lc = h - l1 to FP32 relative
// precision.  Every difference of two stencil points is then a sum of positive gaps (no
// cancellation).  Same formulas as the position form (the differences are the same
// quantities), different rounding.
// ---------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void insert_interface_gaps(const T p[7], T r1, T rc, T l1, T lc, T h, T hf, T hb, T G[6],
                                                      T hs[7])
{
    hs[3] = p[3];
    if (r1 < h) {
        G[3] = r1; G[4] = rc; G[5] = h;
        hs[4] = hf; hs[5] = p[4]; hs[6] = p[5];
    } else {
        G[3] = h; G[4] = h; G[5] = h;
        hs[4] = p[4]; hs[5] = p[5]; hs[6] = p[6];
    }
    if (l1 < h) {
        G[2] = l1; G[1] = lc; G[0] = h;
        hs[2] = hb; hs[1] = p[2]; hs[0] = p[1];
    } else {
        G[2] = h; G[1] = h; G[0] = h;
        hs[2] = p[2]; hs[1] = p[1]; hs[0] = p[0];
    }
}

// differences e[b] - e[a] of six faces from the five gaps between consecutive faces
template <typename T> struct FaceSpan {
    T d01, d12, d23, d34, d45, d02, d13, d24, d35, d03, d14, d25, d04, d15, d05;
    __device__ __forceinline__ explicit FaceSpan(const T g[5])
    {
        d01 = g[0]; d12 = g[1]; d23 = g[2]; d34 = g[3]; d45 = g[4];
        d02 = d01 + d12; d13 = d12 + d23; d24 = d23 + d34; d35 = d34 + d45;
        d03 = d02 + d23; d14 = d13 + d34; d25 = d24 + d45;
        d04 = d03 + d34; d15 = d14 + d45; d05 = d04 + d45;
    }
};

// nu_smoothness on face spans (faces xm25, xm15, xm05, x05, x15, x25 = e[0..5])
template <typename T> __device__ __forceinline__ void nu_smoothness_gaps(const FaceSpan<T> &D, const T u[5], T s[3])
{
    const T um2 = u[0], um1 = u[1], u0 = u[2], u1 = u[3], u2 = u[4];
    const T w = D.d23;
    s[0] = T(4.0) * sqr(w / D.d25) *
           (sqr((u2 - u1) / D.d35) * (T(10.0) * sqr(w) + D.d24 * D.d34) +
            (u2 - u1) * (u0 - u1) / (D.d35 * D.d24) *
                (T(20.0) * sqr(w) + T(2.0) * D.d24 * D.d34 + D.d25 * (D.d34 + D.d24)) +
            sqr((u0 - u1) / D.d24) * (T(10.0) * sqr(w) + (D.d25 + D.d24) * (D.d35 + D.d24)));
    s[1] = T(4.0) * sqr(w / D.d14) *
           (sqr((um1 - u0) / D.d13) * (T(10.0) * sqr(w) + D.d24 * D.d34) +
            (u1 - u0) * (um1 - u0) / (D.d24 * D.d13) * (T(20.0) * sqr(w) - D.d34 * D.d12 - D.d24 * D.d13) +
            sqr((u1 - u0) / D.d24) * (T(10.0) * sqr(w) + D.d12 * D.d13));
    s[2] = T(4.0) * sqr(w / D.d03) *
           (sqr((um2 - um1) / D.d02) * (T(10.0) * sqr(w) + D.d13 * D.d12) +
            (u0 - um1) * (um2 - um1) / (D.d13 * D.d02) *
                (T(20.0) * sqr(w) + T(2.0) * D.d13 * D.d12 + D.d03 * (D.d13 + D.d12)) +
            sqr((u0 - um1) / D.d13) * (T(10.0) * sqr(w) + (D.d03 + D.d13) * (D.d13 + D.d02)));
}

// weno_nonuniform_pair on the gaps G[m] = xs[m+1] - xs[m] and the divided differences
// dd[m] = (hs[m+1] - hs[m]) / G[m]
template <typename T>
__device__ __noinline__ void weno_nonuniform_pair_dd(const T G[6], const T dd[6], T &d_fore, T &d_back)
{
    T u[5], v[3], c[3], s[3];
    {  // forward bias: faces xs[1..6], cells dd[1..5]
        const FaceSpan<T> D(G + 1);
#pragma unroll
        for (int m = 0; m < 5; ++m) u[m] = dd[m + 1];
        const T um2 = u[0], um1 = u[1], u0 = u[2], u1 = u[3], u2 = u[4];
        v[0] = u1 + (u0 - u1) * (T(1.0) + D.d23 / D.d24 + D.d23 / D.d25) + (u2 - u1) * (D.d23 / D.d25) * (D.d24 / D.d35);
        v[1] = u0 + (um1 - u0) * (D.d23 / D.d14) * (D.d24 / D.d13) - (u1 - u0) * (D.d23 / D.d14) * (D.d12 / D.d24);
        v[2] = um1 + (u0 - um1) * (D.d12 / D.d03) * (D.d02 / D.d13) - (um2 - um1) * (D.d12 / D.d03) * (D.d23 / D.d02);
        c[0] = (D.d12 / D.d05) * (D.d02 / D.d15);
        c[1] = (D.d02 / D.d05) * (D.d25 / D.d15) * (T(1.0) + D.d15 / D.d04);
        c[2] = (D.d24 / D.d05) * (D.d25 / D.d04);
        nu_smoothness_gaps(D, u, s);
        d_fore = nu_combine(v, c, s);
    }
    {  // backward bias: faces xs[0..5], cells dd[0..4]
        const FaceSpan<T> D(G);
#pragma unroll
        for (int m = 0; m < 5; ++m) u[m] = dd[m];
        const T um2 = u[0], um1 = u[1], u0 = u[2], u1 = u[3], u2 = u[4];
        v[0] = u1 + (u0 - u1) * (D.d34 / D.d25) * (D.d35 / D.d24) - (u2 - u1) * (D.d34 / D.d25) * (D.d23 / D.d35);
        v[1] = u0 + (u1 - u0) * (D.d23 / D.d14) * (D.d13 / D.d24) - (um1 - u0) * (D.d23 / D.d14) * (D.d34 / D.d13);
        v[2] = um1 + (um2 - um1) * (D.d23 / D.d02) * (D.d13 / D.d03) + (u0 - um1) * (T(1.0) + D.d23 / D.d13 + D.d23 / D.d03);
        c[0] = (D.d03 / D.d05) * (D.d13 / D.d15);
        c[1] = (D.d03 / D.d05) * (D.d35 / D.d15) * (T(1.0) + D.d15 / D.d04);
        c[2] = (D.d34 / D.d05) * (D.d35 / D.d04);
        nu_smoothness_gaps(D, u, s);
        d_back = nu_combine(v, c, s);
    }
}

// eno3_nonuniform_pair on the gaps G[m] = xs[m+1] - xs[m] and the divided differences
// dd[m] = (hs[m+1] - hs[m]) / G[m]
template <typename T>
__device__ __noinline__ void eno3_nonuniform_pair_dd(const T G[6], const T dd[6], T &d_fore, T &d_back)
{
    const T f25 = dd[5], f15 = dd[4], f05 = dd[3], fm05 = dd[2], fm15 = dd[1], fm25 = dd[0];
    T g2 = (f25 - f15) / (G[4] + G[5]);
    T g1 = (f15 - f05) / (G[3] + G[4]);
    T g0 = (f05 - fm05) / (G[2] + G[3]);
    T gm1 = (fm05 - fm15) / (G[1] + G[2]);
    T gm2 = (fm15 - fm25) / (G[0] + G[1]);
    T t15 = (g2 - g1) / (G[3] + G[4] + G[5]);
    T t05 = (g1 - g0) / (G[2] + G[3] + G[4]);
    T tm05 = (g0 - gm1) / (G[1] + G[2] + G[3]);
    T tm15 = (gm1 - gm2) / (G[0] + G[1] + G[2]);
    // x0 - x1m = G[2], x0 - x2m = G[1] + G[2], x0 - x1 = -G[3], x0 - x2 = -(G[3] + G[4])
    T a1 = G[2] * (G[1] + G[2]) * minabs(tm05, tm15);
    T a2 = -(G[2] * G[3]) * minabs(tm05, t05);
    T a = (fabs(gm1) < fabs(g0)) ? a1 : a2;
    T b1 = -(G[2] * G[3]) * minabs(tm05, t05);
    T b2 = G[3] * (G[3] + G[4]) * minabs(t05, t15);
    T b = (fabs(g0) < fabs(g1)) ? b1 : b2;
    d_back = fm05 + minmod(gm1, g0) * G[2] + a;
    d_fore = f05 - minmod(g0, g1) * G[3] + b;
}

// Interface-aware pair of the mixed form: rc / lc are h - r1 / h - l1 as the neighbours
// beyond the crossings store them (read only where r1 / l1 < h).
template <typename T>
__device__ __forceinline__ void interface_pair_gaps(const T p[7], T r1, T rc, T l1, T lc, T h, T hf, T hb, bool eno3,
                                                    T &d_fore, T &d_back)
{
    T G[6], hs[7], dd[6];
    insert_interface_gaps(p, r1, rc, l1, lc, h, hf, hb, G, hs);
#pragma unroll
    for (int m = 0; m < 6; ++m) dd[m] = (hs[m + 1] - hs[m]) / G[m];
    if (eno3)
        eno3_nonuniform_pair_dd(G, dd, d_fore, d_back);
    else
        weno_nonuniform_pair_dd(G, dd, d_fore, d_back);
}

// Godunov |grad phi| for the reinitialization Hamiltonian; `neg` is the mask (phi0 < 0)
// (re_step.cu:382-392).  Per axis max(max(0, D-)^2, min(0, D+)^2) is formed as
// max(0, D-, -D+)^2 (and with both derivatives negated where neg): the squares of non-negative
// numbers keep their order, also when rounded, so the square of the maximum is the maximum
// of the squares, bit for bit, with one square per axis instead of two.  The sums are
// explicitly rounded (no multiply-add contraction), as the maxima between squares and sums
// kept them before.
template <typename T> __device__ __forceinline__ T add_rn(T x, T y);
template <> __device__ __forceinline__ float add_rn<float>(float x, float y) { return __fadd_rn(x, y); }
template <> __device__ __forceinline__ double add_rn<double>(double x, double y) { return __dadd_rn(x, y); }
// square root of the norm: FP32 by the bare PTX sqrt.approx.ftz.f32 (the sums are normal
// or zero; checked bitwise on the GPU against sqrtf of the fast-math build)
template <typename T> __device__ __forceinline__ T norm_root(T x) { return sqrt(x); }
template <> __device__ __forceinline__ float norm_root<float>(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
template <typename T>
__device__ __forceinline__ T godunov_norm(bool neg, T xR, T xL, T yF, T yB, T zU, T zD)
{
    const T z = T(0);
    T a, b, c;
    if (neg) {
        a = vmax(z, vmax(-xL, xR));
        b = vmax(z, vmax(-yB, yF));
        c = vmax(z, vmax(-zD, zU));
    } else {
        a = vmax(z, vmax(xL, -xR));
        b = vmax(z, vmax(yB, -yF));
        c = vmax(z, vmax(zD, -zU));
    }
    return norm_root(add_rn(add_rn(sqr(a), sqr(b)), sqr(c)));
}

// Upwind transport term sum_a min(0,v_a) D+_a + max(0,v_a) D-_a (extend_step.cu:121-123).
template <typename T>
__device__ __forceinline__ T upwind_dot(T vx, T vy, T vz, T xR, T xL, T yF, T yB, T zU, T zD)
{
    const T z = T(0);
    return vmin(z, vx) * xR + vmax(z, vx) * xL + vmin(z, vy) * yF + vmax(z, vy) * yB + vmin(z, vz) * zU +
           vmax(z, vz) * zD;
}

// Degree-5 value of the line at the crossing (sixth_interp, boundary_interpolant.cu:78-99)
// and the cubic one (cubic_interp, wenork3_extend.cu:296-328); double throughout.
__device__ inline void crossing_quintic(const double p[7], double dis_f, double dis_b, double h, double &cf,
                                        double &cb)
{
    cf = 0.0;
    cb = 0.0;
    if (dis_f < h) {
        double xs[6] = {h, 2 * h, 3 * h, 4 * h, 5 * h, 6 * h};
        double a[6];
        lagrange_monomial<5>(xs, p + 1, a);
        cf = poly_eval<5>(a, 3 * h + dis_f);
    }
    if (dis_b < h) {
        double xs[6] = {0.0, h, 2 * h, 3 * h, 4 * h, 5 * h};
        double a[6];
        lagrange_monomial<5>(xs, p, a);
        cb = poly_eval<5>(a, 3 * h - dis_b);
    }
}

__device__ __forceinline__ void cubic_fit(double v0, double v1, double v2, double v3, double h, double a[4])
{
    a[0] = v0;
    a[1] = (3.0 * (v1 - v0) - 3.0 / 2.0 * (v2 - v0) + 1.0 / 3.0 * (v3 - v0)) / h;
    a[2] = (-5.0 / 2.0 * (v1 - v0) + 2.0 * (v2 - v0) - 1.0 / 2.0 * (v3 - v0)) / (h * h);
    a[3] = (1.0 / 2.0 * (v1 - v0) - 1.0 / 2.0 * (v2 - v0) + 1.0 / 6.0 * (v3 - v0)) / pow_cr<3>(h);
}

__device__ inline void crossing_cubic(const double p[7], double dis_f, double dis_b, double h, double &cf,
                                      double &cb)
{
    cf = 0.0;
    cb = 0.0;
    double a[4];
    if (dis_f < h) {
        cubic_fit(p[2], p[3], p[4], p[5], h, a);
        double t = h + dis_f;
        cf = a[0] + a[1] * t + a[2] * (t * t) + a[3] * pow_cr<3>(t);
    }
    if (dis_b < h) {
        cubic_fit(p[1], p[2], p[3], p[4], h, a);
        double t = 2 * h - dis_b;
        cb = a[0] + a[1] * t + a[2] * (t * t) + a[3] * pow_cr<3>(t);
    }
}

// ---------------------------------------------------------------------------------------
// Packed FP32 pairs (sm_100+ dual-lane FMA/MUL/ADD): the backward and forward WENO5
// reconstructions of a node are the same arithmetic on mirrored differences, so the
// mixed-precision form evaluates them as the .x (backward) and .y (forward) lanes of
// float2 operations.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 rcp2(float2 b) { return f2(rcp_ftz(b.x), rcp_ftz(b.y)); }
__device__ __forceinline__ float2 fdiv2(float2 a, float2 b) { return mul2(a, rcp2(b)); }

// Candidate values of the three stencils for packed differences u1..u5.
__device__ __forceinline__ void weno5_candidates2(float2 u1, float2 u2, float2 u3, float2 u4, float2 u5, float2 &q1,
                                                  float2 &q2, float2 &q3)
{
    q1 = fma2(f2s(1.f / 3.f), u1, fma2(f2s(-7.f / 6.f), u2, mul2(f2s(11.f / 6.f), u3)));
    q2 = fma2(f2s(-1.f / 6.f), u2, fma2(f2s(5.f / 6.f), u3, mul2(f2s(1.f / 3.f), u4)));
    q3 = fma2(f2s(1.f / 3.f), u3, fma2(f2s(5.f / 6.f), u4, mul2(f2s(-1.f / 6.f), u5)));
}

// Reciprocal weights 1/(S_k + eps2)^2 of packed windows.
__device__ __forceinline__ void weno5_weights2(float2 u1, float2 u2, float2 u3, float2 u4, float2 u5, float2 eps2,
                                               float2 &r1, float2 &r2, float2 &r3)
{
    const float2 c13 = f2s(13.f / 12.f), c14 = f2s(0.25f);
    const float2 t1 = fma2(f2s(-2.f), u2, add2(u1, u3));
    const float2 t2 = fma2(f2s(-4.f), u2, fma2(f2s(3.f), u3, u1));
    const float2 t3 = fma2(f2s(-2.f), u3, add2(u2, u4));
    const float2 t4 = fma2(f2s(-1.f), u4, u2);
    const float2 t5 = fma2(f2s(-2.f), u4, add2(u3, u5));
    const float2 t6 = fma2(f2s(-4.f), u4, fma2(f2s(3.f), u3, u5));
    const float2 s1 = fma2(c13, mul2(t1, t1), mul2(c14, mul2(t2, t2)));
    const float2 s2 = fma2(c13, mul2(t3, t3), mul2(c14, mul2(t4, t4)));
    const float2 s3 = fma2(c13, mul2(t5, t5), mul2(c14, mul2(t6, t6)));
    const float2 e1 = add2(s1, eps2), e2 = add2(s2, eps2), e3 = add2(s3, eps2);
    r1 = rcp2(mul2(e1, e1));
    r2 = rcp2(mul2(e2, e2));
    r3 = rcp2(mul2(e3, e3));
}

// Weighted combination sum(d_k r_k q_k) / sum(d_k r_k), d = (0.1, 0.6, 0.3).
__device__ __forceinline__ float2 weno5_combine2(float2 q1, float2 q2, float2 q3, float2 r1, float2 r2, float2 r3)
{
    const float2 a1 = mul2(f2s(0.1f), r1), a2 = mul2(f2s(0.6f), r2), a3 = mul2(f2s(0.3f), r3);
    return fdiv2(fma2(a1, q1, fma2(a2, q2, mul2(a3, q3))), add2(a1, add2(a2, a3)));
}

// Backward (.x) and forward (.y) WENO5 derivatives from the seven line values.
__device__ __forceinline__ void weno5_pair_fast2(const float p[7], float inv_h, float eps2, float &d_fore,
                                                 float &d_back)
{
    float u[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) u[m] = p[m + 1] - p[m];
    // backward window u0..u4, forward window u5..u1
    const float2 U1 = f2(u[0], u[5]), U2 = f2(u[1], u[4]), U3 = f2(u[2], u[3]), U4 = f2(u[3], u[2]),
                 U5 = f2(u[4], u[1]);
    float2 q1, q2, q3, r1, r2, r3;
    weno5_candidates2(U1, U2, U3, U4, U5, q1, q2, q3);
    weno5_weights2(U1, U2, U3, U4, U5, f2s(eps2), r1, r2, r3);
    const float2 d = mul2(weno5_combine2(q1, q2, q3, r1, r2, r3), f2s(inv_h));
    d_back = d.x;
    d_fore = d.y;
}

// Upwind WENO5 derivatives of two lines as the two lanes of one packed evaluation: lane
// .x takes the backward derivative of line a where back_a holds and its forward derivative
// (the mirrored window) otherwise, lane .y the same for line b.  For a transport term
// min(0,v) D+ + max(0,v) D- only the derivative on the upwind side is ever multiplied by
// a nonzero speed, so one lane per axis replaces the pair.
__device__ __forceinline__ float2 weno5_upwind2(const float pa[7], bool back_a, const float pb[7], bool back_b,
                                                float2 inv_h, float2 eps2)
{
    float ua[6], ub[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
        ua[m] = pa[m + 1] - pa[m];
        ub[m] = pb[m + 1] - pb[m];
    }
    // backward window u0..u4, forward window u5..u1
    float2 U[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) U[m] = f2(back_a ? ua[m] : ua[5 - m], back_b ? ub[m] : ub[5 - m]);
    float2 q1, q2, q3, r1, r2, r3;
    weno5_candidates2(U[0], U[1], U[2], U[3], U[4], q1, q2, q3);
    weno5_weights2(U[0], U[1], U[2], U[3], U[4], eps2, r1, r2, r3);
    return mul2(weno5_combine2(q1, q2, q3, r1, r2, r3), inv_h);
}

// Crossing values for the mixed-precision form: the same interpolating polynomials
// (degree 5 through six nodes, or the cubic through four) evaluated in Lagrange product
// form at the normalised abscissa t (node spacing 1), in FP64 on the promoted FP32 values.
// The reference builds monomial coefficients in FP64 (boundary_interpolant.cu:78-99,
// wenork3_extend.cu:296-328); the product form is the better-conditioned evaluation of the
// same polynomial, and reproduces the node values exactly at the nodes.
template <int NPT, typename T>
__device__ __forceinline__ T lagrange_equispaced(const T *y, T t)
{
    // nodes 0..NPT-1; weight_m = prod_{q != m} (t - q) / prod_{q != m} (m - q)
    T d[NPT], pre[NPT], suf[NPT];
#pragma unroll
    for (int q = 0; q < NPT; ++q) d[q] = t - (T)q;
    pre[0] = T(1);
#pragma unroll
    for (int q = 1; q < NPT; ++q) pre[q] = pre[q - 1] * d[q - 1];
    suf[NPT - 1] = T(1);
#pragma unroll
    for (int q = NPT - 2; q >= 0; --q) suf[q] = suf[q + 1] * d[q + 1];
    T v = T(0);
#pragma unroll
    for (int m = 0; m < NPT; ++m) {
        T den = T(1);
#pragma unroll
        for (int q = 0; q < NPT; ++q)
            if (q != m) den *= (T)(m - q);
        v += y[m] * (pre[m] * suf[m]) * (T(1) / den);
    }
    return v;
}

// ---------------------------------------------------------------------------------------
// ENORK2: second-order ENO derivatives with the sub-cell fix (Min 2010), on the five
// values p[1..5] of a 7-point line centred at p[3]
// ---------------------------------------------------------------------------------------

// Forward (sR) and backward (sL) derivatives at p[3]; where the interface cuts the cell
// (r1 / l1 differs from h) the one-sided difference runs to the interface, whose value is
// hf / hb (0 for reinitialization, the crossing value for extension).  eno_derivative,
// boundary_correction.cu:81-101; eno_derivative_field, enork2_extend.cu:56-75.
template <typename T>
__device__ __forceinline__ void eno2_pair(const T p[7], T r1, T l1, T h, T hf, T hb, T &sR, T &sL)
{
    const T v4 = p[1], v1 = p[2], v0 = p[3], v2 = p[4], v3 = p[5];
    const T h2 = sqr(h);
    const T p2 = v1 - T(2.0) * v0 + v2;
    const T p2r = v0 - T(2.0) * v2 + v3;
    T p2m = T(0.5) * minmod(p2, p2r) / h2;
    const T vr = (r1 == h) ? v2 : hf;
    sR = (vr - v0) / r1 - r1 * p2m;
    const T p2l = v0 - T(2.0) * v1 + v4;
    p2m = T(0.5) * minmod(p2, p2l) / h2;
    const T vl = (l1 == h) ? v1 : hb;
    sL = (v0 - vl) / l1 + l1 * p2m;
}

// The ENO derivative toward the side whose neighbour value (0 across the interface) is
// smaller in magnitude (upwind_normal_point, enork2_extend.cu:82-100).
template <typename T> __device__ __forceinline__ T eno2_upwind(const T p[7], T r1, T l1, T h)
{
    T sR, sL;
    eno2_pair(p, r1, l1, h, T(0), T(0), sR, sL);
    const T vr = (r1 == h) ? p[4] : T(0);
    const T vl = (l1 == h) ? p[2] : T(0);
    return (fabs(vr) < fabs(vl)) ? sR : sL;
}

// Value at the crossing of the quadratic ENO interpolant of the cut cell, 0 where the
// cell is not cut (cubic_eno_interp, enork2_extend.cu:144-172).
template <typename T>
__device__ __forceinline__ void eno2_crossing(const T p[7], T dis_f, T dis_b, T h, T &cf, T &cb)
{
    const T v4 = p[1], v1 = p[2], v0 = p[3], v2 = p[4], v3 = p[5];
    const T h2 = sqr(h);
    cf = T(0);
    cb = T(0);
    if (dis_f != h) {
        const T p2 = v2 - T(2.0) * v0 + v1;
        const T p2r = v3 - T(2.0) * v2 + v0;
        const T c2 = T(0.5) * minmod(p2, p2r) / h2;
        const T c1 = (v2 - v0) / h;
        const T c0 = (v2 + v0) / T(2) - c2 * h2 / T(4);
        const T x = dis_f - h / T(2);
        cf = c2 * x * x + c1 * x + c0;
    }
    if (dis_b != h) {
        const T p2 = v2 - T(2.0) * v0 + v1;
        const T p2l = v0 - T(2.0) * v1 + v4;
        const T c2 = T(0.5) * minmod(p2, p2l) / h2;
        const T c1 = (v0 - v1) / h;
        const T c0 = (v1 + v0) / T(2) - c2 * h2 / T(4);
        const T x = h / T(2) - dis_b;
        cb = c2 * x * x + c1 * x + c0;
    }
}

// Distance from the node at L.c to the interface between it and its +1 neighbour along
// L by the quadratic ENO fit alone (the ENORK2 boundary_correction,
// boundary_correction.cu:104-146), double arithmetic on the promoted samples.
template <typename T>
__device__ __forceinline__ double eno2_fore_distance(const T *__restrict__ f, const AxisLine &L, double h)
{
    const double a = (double)__ldg(f + L.base + (long long)clampi(L.c - 1, L.n) * L.stride);
    const double b = (double)__ldg(f + L.base + (long long)L.c * L.stride);
    const double c = (double)__ldg(f + L.base + (long long)clampi(L.c + 1, L.n) * L.stride);
    const double d = (double)__ldg(f + L.base + (long long)clampi(L.c + 2, L.n) * L.stride);
    return eno2_distance(a, b, c, d, h);
}

}  // namespace vsl
