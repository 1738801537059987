// vsl_relax.cuh -- the pieces of the single-phase relaxation step of the vesicle driver
// (p00_test_singlephase_relax.m:60-196) that are not level-set operators of their own:
// the periodic Laplacian of SD.GD3 (GD3.m:344-346, circshift neighbours), the bending
// normal speed, the FP64 surface integrals of the tension/pressure solve, the 2x2 solve
// itself, the normal speed and the explicit update.  Templated on the field type;
// included by vsl_relax_f64.cu (no multiply-add contraction, the reference's rounding)
// and vsl_relax_f32.cu (mixed form).
#pragma once

#include <cmath>
#include <limits>

#include "vsl_internal.h"

namespace vsl {
namespace {

constexpr int RNT = BX * BY;
constexpr int RNW = RNT / 32;

__device__ __forceinline__ bool relax_node(const Grid &g, int &i, int &j, int &k, long long &c)
{
    i = blockIdx.x * BX + threadIdx.x;
    j = blockIdx.y * BY + threadIdx.y;
    k = blockIdx.z;
    if (i >= g.rows || j >= g.cols) return false;
    c = node_index(g, i, j, k);
    return true;
}

__device__ __forceinline__ long long relax_block() { return blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z); }

__device__ __forceinline__ double relax_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// GD3.Laplacian: (Fxx + Fyy) + Fzz with Fxx = (F(j+1) - 2F + F(j-1)) / Dx^2 and periodic
// neighbours (circshift, GD3.m:111-116)
template <typename T>
__device__ __forceinline__ T periodic_laplacian(const T *__restrict__ f, const Grid &g, int i, int j, int k, long long c,
                                                T dx2, T dy2, T dz2)
{
    const int jp = j + 1 == g.cols ? 0 : j + 1, jm = j == 0 ? g.cols - 1 : j - 1;
    const int ip = i + 1 == g.rows ? 0 : i + 1, im = i == 0 ? g.rows - 1 : i - 1;
    const int kp = k + 1 == g.pges ? 0 : k + 1, km = k == 0 ? g.pges - 1 : k - 1;
    const T fc = __ldg(f + c);
    const T fxx = (__ldg(f + node_index(g, i, jp, k)) - T(2) * fc + __ldg(f + node_index(g, i, jm, k))) / dx2;
    const T fyy = (__ldg(f + node_index(g, ip, j, k)) - T(2) * fc + __ldg(f + node_index(g, im, j, k))) / dy2;
    const T fzz = (__ldg(f + node_index(g, i, j, kp)) - T(2) * fc + __ldg(f + node_index(g, i, j, km))) / dz2;
    return fxx + fyy + fzz;
}

template <typename T>
__global__ void __launch_bounds__(RNT) k_laplacian(const T *__restrict__ f, T *__restrict__ out, Grid g, T dx2, T dy2,
                                                   T dz2)
{
    int i, j, k;
    long long c;
    if (!relax_node(g, i, j, k, c)) return;
    out[c] = periodic_laplacian(f, g, i, j, k, c, dx2, dy2, dz2);
}

// GD3.Gradient (GD3.m:314-318): Fx = (F(oXo) - F(oxo)) / (2 Dx), Fy, Fz alike (GD3.m:218-240),
// with the periodic neighbours of the Laplacian
template <typename T>
__global__ void __launch_bounds__(RNT) k_gradient(const T *__restrict__ f, T *__restrict__ fx, T *__restrict__ fy,
                                                  T *__restrict__ fz, Grid g, T two_dx, T two_dy, T two_dz)
{
    int i, j, k;
    long long c;
    if (!relax_node(g, i, j, k, c)) return;
    const int jp = j + 1 == g.cols ? 0 : j + 1, jm = j == 0 ? g.cols - 1 : j - 1;
    const int ip = i + 1 == g.rows ? 0 : i + 1, im = i == 0 ? g.rows - 1 : i - 1;
    const int kp = k + 1 == g.pges ? 0 : k + 1, km = k == 0 ? g.pges - 1 : k - 1;
    fx[c] = (__ldg(f + node_index(g, i, jp, k)) - __ldg(f + node_index(g, i, jm, k))) / two_dx;
    fy[c] = (__ldg(f + node_index(g, ip, j, k)) - __ldg(f + node_index(g, im, j, k))) / two_dy;
    fz[c] = (__ldg(f + node_index(g, i, j, kp)) - __ldg(f + node_index(g, i, j, km))) / two_dz;
}

// NormalSpeedBend = Kappa * (Lap H + 0.5 H (H^2 - 4 K) + 2 c0 K - 0.5 c0^2 H)
// (p00_test_singlephase_relax.m:80-84), H the extended mean curvature, K the Gaussian
// curvature, c0 the spontaneous curvature
template <typename T>
__global__ void __launch_bounds__(RNT) k_bending_speed(const T *__restrict__ H, const T *__restrict__ K,
                                                       T *__restrict__ out, Grid g, T dx2, T dy2, T dz2, T kappa,
                                                       T two_c0, T half_c0sq)
{
    int i, j, k;
    long long c;
    if (!relax_node(g, i, j, k, c)) return;
    const T lap = periodic_laplacian(H, g, i, j, k, c, dx2, dy2, dz2);
    const T h = __ldg(H + c), kk = __ldg(K + c);
    out[c] = kappa * (lap + T(0.5) * h * (h * h - T(4) * kk) + two_c0 * kk - half_c0sq * h);
}

// Per-block FP64 partial sums over the band |F| < 2 Ds of the surface integrals
// sum((f .* DiracDelta) .* FGradMag) (SDF3.m:82-85):
//   MODE 0: f = H^2, H, H .* NSB, NSB   (c11, c12 and the integrals of s1, s2)
//   MODE 1: f = (H - c0)^2              (the bending energy)
// thr: 2 Ds rounded up to T, so that |F| < thr in T is the FP64 test.
template <typename T, int MODE>
__global__ void __launch_bounds__(RNT) k_relax_moments(const T *__restrict__ F, const T *__restrict__ H,
                                                       const T *__restrict__ nsb, const T *__restrict__ delta,
                                                       const T *__restrict__ gmag, T thr, double c0, Grid g,
                                                       double *__restrict__ partials)
{
    constexpr int NC = MODE == 0 ? 4 : 1;
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z;
    double m[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) m[q] = 0.0;
    bool in = false;
    if (i < g.rows && j < g.cols) {
        const long long c = node_index(g, i, j, k);
        if (fabs(__ldg(F + c)) < thr) {
            in = true;
            const double h = (double)__ldg(H + c), d = (double)__ldg(delta + c), gm = (double)__ldg(gmag + c);
            if (MODE == 0) {
                const double s = (double)__ldg(nsb + c);
                m[0] = ((h * h) * d) * gm;
                m[1] = (h * d) * gm;
                m[NC > 2 ? 2 : 0] = ((h * s) * d) * gm;
                m[NC > 3 ? 3 : 0] = (s * d) * gm;
            } else {
                const double e = h - c0;
                m[0] = ((e * e) * d) * gm;
            }
        }
    }
    __shared__ double sm[NC][RNW];
    const int t = threadIdx.y * BX + threadIdx.x;
    const bool any = __any_sync(0xffffffffu, in);
#pragma unroll
    for (int q = 0; q < NC; ++q) {
        double v = any ? relax_warp_sum(m[q]) : 0.0;
        if ((t & 31) == 0) sm[q][t >> 5] = v;
    }
    __syncthreads();
    if (t == 0) {
        const long long b = relax_block();
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            double a = 0.0;
            for (int w = 0; w < RNW; ++w) a += sm[q][w];
            partials[(long long)NC * b + q] = a;
        }
    }
}

// Tension and pressure from TP = [c11, c12; c12, A0] \ [s1; s2] (p00:96-109) with
//   s1 = int(H NSB) - (A0 - A) / Dt,   s2 = int(NSB) + (V0 - V) / Dt,
// by Gaussian elimination with partial pivoting (the LU of a 2x2 backslash).
// mom: the four integrals; av: area, volume at the step's start; dt: the time step.
__global__ void k_tension_pressure(const double *__restrict__ mom, const double *__restrict__ av,
                                   const double *__restrict__ dt, double A0, double V0, double *__restrict__ tp)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double c11 = mom[0], c12 = mom[1], c21 = mom[1], c22 = A0;
    const double s1 = mom[2] - (A0 - av[0]) / dt[0];
    const double s2 = mom[3] + (V0 - av[1]) / dt[0];
    double a11 = c11, a12 = c12, a21 = c21, a22 = c22, b1 = s1, b2 = s2;
    if (fabs(a21) > fabs(a11)) {
        double t;
        t = a11; a11 = a21; a21 = t;
        t = a12; a12 = a22; a22 = t;
        t = b1; b1 = b2; b2 = t;
    }
    const double l = a21 * (1.0 / a11);
    const double u22 = a22 - l * a12;
    const double y2 = b2 - l * b1;
    const double x2 = y2 / u22;
    const double x1 = (b1 - a12 * x2) / a11;
    tp[0] = x1;  // tension
    tp[1] = x2;  // pressure
}

// normalSpeed = (Tension * H - NSB + Pressure) .* FGradMag (p00:114)
template <typename T>
__global__ void __launch_bounds__(RNT) k_normal_speed(const T *__restrict__ H, const T *__restrict__ nsb,
                                                      const T *__restrict__ gmag, const double *__restrict__ tp,
                                                      T *__restrict__ out, Grid g)
{
    int i, j, k;
    long long c;
    if (!relax_node(g, i, j, k, c)) return;
    const T ten = (T)__ldg(tp), pre = (T)__ldg(tp + 1);
    out[c] = (ten * __ldg(H + c) - __ldg(nsb + c) + pre) * __ldg(gmag + c);
}

// F = F - Dt * v (p00:119)
template <typename T>
__global__ void __launch_bounds__(RNT) k_euler(T *__restrict__ F, const T *__restrict__ v, const double *__restrict__ dt,
                                               Grid g)
{
    int i, j, k;
    long long c;
    if (!relax_node(g, i, j, k, c)) return;
    F[c] = F[c] - (T)__ldg(dt) * __ldg(v + c);
}

// the smallest T not below x: |v| < relax_round_up<T>(x) in T  <=>  (double)|v| < x
template <typename T> T relax_round_up(double x);
template <> inline double relax_round_up<double>(double x) { return x; }
template <> inline float relax_round_up<float>(double x)
{
    float r = (float)x;
    if ((double)r < x) r = std::nextafter(r, std::numeric_limits<float>::infinity());
    return r;
}

}  // namespace

// the divisors 2 Dx, 2 Dy, 2 Dz formed in FP64 (GD3.m:219) and rounded once to T
template <typename T> cudaError_t launch_gradient(const T *f, T *fx, T *fy, T *fz, const Grid &g, cudaStream_t s)
{
    k_gradient<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(f, fx, fy, fz, g, (T)(2 * g.dx), (T)(2 * g.dy),
                                                       (T)(2 * g.dz));
    return cudaGetLastError();
}

template <typename T> cudaError_t launch_laplacian(const T *f, T *out, const Grid &g, cudaStream_t s)
{
    k_laplacian<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(f, out, g, (T)(g.dx * g.dx), (T)(g.dy * g.dy),
                                                        (T)(g.dz * g.dz));
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_bending_speed(const T *H, const T *K, T *out, const Grid &g, double kappa, double c0,
                                 cudaStream_t s)
{
    k_bending_speed<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(H, K, out, g, (T)(g.dx * g.dx), (T)(g.dy * g.dy),
                                                            (T)(g.dz * g.dz), (T)kappa, (T)(2. * c0),
                                                            (T)(0.5 * (c0 * c0)));
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_relax_moments(const T *F, const T *H, const T *nsb, const T *delta, const T *gmag, double band,
                                 double c0, bool energy, const Grid &g, double *partials, int *nblocks, cudaStream_t s)
{
    const dim3 gr = node_grid(g);
    if (nblocks) *nblocks = (int)((long long)gr.x * gr.y * gr.z);
    if (energy)
        k_relax_moments<T, 1><<<gr, dim3(BX, BY), 0, s>>>(F, H, nsb, delta, gmag, relax_round_up<T>(band), c0, g,
                                                          partials);
    else
        k_relax_moments<T, 0><<<gr, dim3(BX, BY), 0, s>>>(F, H, nsb, delta, gmag, relax_round_up<T>(band), c0, g,
                                                          partials);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_normal_speed(const T *H, const T *nsb, const T *gmag, const double *tp, T *out, const Grid &g,
                                cudaStream_t s)
{
    k_normal_speed<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(H, nsb, gmag, tp, out, g);
    return cudaGetLastError();
}

template <typename T> cudaError_t launch_euler(T *F, const T *v, const double *dt, const Grid &g, cudaStream_t s)
{
    k_euler<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(F, v, dt, g);
    return cudaGetLastError();
}

#define VSL_INSTANTIATE_RELAX(T)                                                                                   \
    template cudaError_t launch_laplacian<T>(const T *, T *, const Grid &, cudaStream_t);                          \
    template cudaError_t launch_gradient<T>(const T *, T *, T *, T *, const Grid &, cudaStream_t);                 \
    template cudaError_t launch_bending_speed<T>(const T *, const T *, T *, const Grid &, double, double,          \
                                                 cudaStream_t);                                                    \
    template cudaError_t launch_relax_moments<T>(const T *, const T *, const T *, const T *, const T *, double,    \
                                                 double, bool, const Grid &, double *, int *, cudaStream_t);       \
    template cudaError_t launch_normal_speed<T>(const T *, const T *, const T *, const double *, T *, const Grid &, \
                                                cudaStream_t);                                                     \
    template cudaError_t launch_euler<T>(T *, const T *, const double *, const Grid &, cudaStream_t);

}  // namespace vsl
