// vsl_toolbox.cuh -- calculus toolbox fused with the FP64 area/volume reductions and the
// band maximum of the normal speed, templated on the field type.  Included by
// vsl_toolbox.cu (the FP64 plain form, compiled without multiply-add contraction so that
// it rounds like the reference) and vsl_toolbox_f32.cu (the FP32 mixed form, fast
// division); all reductions in a fixed order (per-block warp-shuffle trees, then one
// block summing the block partials in index order), so a result is bitwise reproducible
// for a given grid.
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>
#include <type_traits>

#include "vsl_internal.h"

namespace vsl {
namespace {

constexpr int NT = BX * BY;  // threads per node block
constexpr int NW = NT / 32;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ long long block_linear() { return blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z); }

// set_calculus_toolbox (set_calculus_toolbox.cu:9-107) in the field's precision T (the
// plain form is FP64 throughout; the mixed form computes these stencils in FP32), with
// HPrimal = max(F, 0) formed on the fly (GPUsetCalculusToolBox.m:4); per block the FP64
// sums of DiracDelta over |F| < 2Ds and of 1 - Heaviside over F < 2Ds (SDF3.m:73-80).
template <typename T> __device__ __forceinline__ T cube(T x);
template <> __device__ __forceinline__ double cube<double>(double x) { return pow_cr<3>(x); }
template <> __device__ __forceinline__ float cube<float>(float x) { return x * x * x; }
template <typename T> __device__ __forceinline__ T fourth(T x);
template <> __device__ __forceinline__ double fourth<double>(double x) { return pow_cr<4>(x); }
template <> __device__ __forceinline__ float fourth<float>(float x) { return (x * x) * (x * x); }

// reciprocals of the spacings for the mixed form: FP64 for its area and volume terms, FP32
// for its stencils
struct Recips {
    double i2x, i2y, i2z, ixx, iyy, izz;  // 1 / (2 d), 1 / d^2 per axis
    float f2x, f2y, f2z, fxx, fyy, fzz, f4ds;  // the same in FP32, and 1 / (4 Ds^2)
};

// The FP64 area and volume terms of one band node of the mixed form from its seven FP32
// values v[0..6] (centre, x+, x-, y+, y-, z+, z-) and v[7] != 0 where the node is in the
// area band: FP32 quotients and second differences carry a relative error of ~1e-7 per
// node that does not average out in the sums (4e-8 of the area at 256^3), so the terms are
// FP64 on the promoted values.  FP64 divisions and square roots are slow on this GPU:
// reciprocals of the spacings from the host, |grad|^2 clamped instead of |grad|, one
// division.
__device__ __forceinline__ void band_terms_f64(const float v[8], const Recips &rc, double &area, double &vol,
                                               int &units)
{
    const double c0 = v[0], xp = v[1], xm = v[2], yp = v[3], ym = v[4], zp = v[5], zm = v[6];
    const double gx = (xp - xm) * rc.i2x, gy = (yp - ym) * rc.i2y, gz = (zp - zm) * rc.i2z;
    const double gg = fmax(gx * gx + gy * gy + gz * gz, 1e-28);
    const double l = (xp - 2 * c0 + xm) * rc.ixx + (yp - 2 * c0 + ym) * rc.iyy + (zp - 2 * c0 + zm) * rc.izz;
    const double q0 = fmax(c0, 0.0);
    const double qxp = fmax(xp, 0.0), qxm = fmax(xm, 0.0), qyp = fmax(yp, 0.0), qym = fmax(ym, 0.0);
    const double qzp = fmax(zp, 0.0), qzm = fmax(zm, 0.0);
    const double d = (qxp - qxm) * rc.i2x * gx + (qyp - qym) * rc.i2y * gy + (qzp - qzm) * rc.i2z * gz;
    const double pl = (qxp - 2 * q0 + qxm) * rc.ixx + (qyp - 2 * q0 + qym) * rc.iyy + (qzp - 2 * q0 + qzm) * rc.izz;
    const double igg = 1.0 / gg;
    const double h64 = d * igg;
    if (v[7] != 0.f) area += (pl - d * l * igg) * igg;
    if (h64 == 0.0) {
        units += 1;
    } else {
        const double v1 = 1 - h64;
        if (v1 == 1.0)
            units += 1;
        else
            vol += v1;
    }
}

// One node of the mixed form's toolbox: the expressions of toolbox_point in FP32 with the
// divisions by the spacings as products with their FP32 reciprocals and one reciprocal of
// |grad F| (the reference's quotients, rounded differently within a few ulp); the fields
// that only an output needs (Gaussian curvature, Heaviside, Dirac delta) are formed only
// when that output is requested.  Returns whether the node carries FP64 area and volume
// terms (a node of the volume band, F < 2 Ds, with a positive value among its seven), with
// the inputs of band_terms_f64 in v; a node of the volume band without a positive value
// has a volume term of exactly 1 (Heaviside 0, Dirac 0) and is counted in units here.
template <class Get>
__device__ __forceinline__ bool toolbox_point_f32(Get F, int i, int j, int k, int im, int ip, int jm, int jp, int km,
                                                  int kp, long long c, const ToolboxOut<float> &o, float thr2ds,
                                                  const Recips &rc, float v[8], int &units)
{
    const float fc = F(i, j, k);
    const float fxp = F(i, jp, k), fxm = F(i, jm, k), fyp = F(ip, j, k), fym = F(im, j, k);
    const float fzp = F(i, j, kp), fzm = F(i, j, km);
    const float fx = (fxp - fxm) * rc.f2x, fy = (fyp - fym) * rc.f2y, fz = (fzp - fzm) * rc.f2z;
    const float gm = vmax(sqrtf(fx * fx + fy * fy + fz * fz), 1e-14f);
    const float ig = rcp_ftz(gm);  // gm >= 1e-14: a normal number
    const bool pos =
        fc > 0.f || fxp > 0.f || fxm > 0.f || fyp > 0.f || fym > 0.f || fzp > 0.f || fzm > 0.f;
    const bool need = fc < thr2ds && pos;
    if (need) {
        v[0] = fc;
        v[1] = fxp;
        v[2] = fxm;
        v[3] = fyp;
        v[4] = fym;
        v[5] = fzp;
        v[6] = fzm;
        v[7] = fabsf(fc) < thr2ds ? 1.f : 0.f;
    } else if (fc < thr2ds) {
        units += 1;
    }
    if (o.f[0]) o.f[0][c] = fx;
    if (o.f[1]) o.f[1][c] = fy;
    if (o.f[2]) o.f[2][c] = fz;
    if (o.f[3]) o.f[3][c] = gm;
    if (o.f[4]) o.f[4][c] = fx * ig;
    if (o.f[5]) o.f[5][c] = fy * ig;
    if (o.f[6]) o.f[6][c] = fz * ig;
    const bool second = o.f[7] || o.f[8] || o.f[9] || o.f[10] || o.f[11] || o.f[12] || o.f[13] || o.f[14] ||
                        o.f[15] || o.f[17];
    if (!second && !o.f[16]) return need;
    const float fxx = (fxp - 2.f * fc + fxm) * rc.fxx;
    const float fyy = (fyp - 2.f * fc + fym) * rc.fyy;
    const float fzz = (fzp - 2.f * fc + fzm) * rc.fzz;
    const float lap = fxx + fyy + fzz;
    const float ig2 = ig * ig;
    if (second) {
        const float fxy = (F(ip, jp, k) + F(im, jm, k) - F(ip, jm, k) - F(im, jp, k)) * rc.f4ds;
        const float fyz = (F(ip, j, kp) + F(im, j, km) - F(ip, j, km) - F(im, j, kp)) * rc.f4ds;
        const float fzx = (F(i, jp, kp) + F(i, jm, km) - F(i, jp, km) - F(i, jm, kp)) * rc.f4ds;
        if (o.f[7]) o.f[7][c] = fxx;
        if (o.f[8]) o.f[8][c] = fyy;
        if (o.f[9]) o.f[9][c] = fzz;
        if (o.f[10]) o.f[10][c] = fxy;
        if (o.f[11]) o.f[11][c] = fyz;
        if (o.f[12]) o.f[12][c] = fzx;
        if (o.f[13]) o.f[13][c] = lap;
        if (o.f[14]) {
            const float r1 = fxx * fx + fxy * fy + fzx * fz;
            const float r2 = fxy * fx + fyy * fy + fyz * fz;
            const float r3 = fzx * fx + fyz * fy + fzz * fz;
            o.f[14][c] = -lap * ig + (fx * r1 + fy * r2 + fz * r3) * (ig2 * ig);
        }
        if (o.f[15]) {
            const float q1 = (fyy * fzz - fyz * fyz) * fx + (fzx * fyz - fxy * fzz) * fy + (fxy * fyz - fzx * fyy) * fz;
            const float q2 = (fyz * fzx - fxy * fzz) * fx + (fxx * fzz - fzx * fzx) * fy + (fzx * fxy - fxx * fyz) * fz;
            const float q3 = (fxy * fyz - fyy * fzx) * fx + (fzx * fxy - fxx * fyz) * fy + (fxx * fyy - fxy * fxy) * fz;
            o.f[15][c] = (fx * q1 + fy * q2 + fz * q3) * (ig2 * ig2);
        }
    }
    if (o.f[16] || o.f[17]) {
        auto H = [&](int a, int b, int e) { return vmax(F(a, b, e), 0.f); };
        const float hc = vmax(fc, 0.f);
        const float hxp = H(i, jp, k), hxm = H(i, jm, k), hyp = H(ip, j, k), hym = H(im, j, k);
        const float hzp = H(i, j, kp), hzm = H(i, j, km);
        const float dot = (hxp - hxm) * rc.f2x * fx + (hyp - hym) * rc.f2y * fy + (hzp - hzm) * rc.f2z * fz;
        if (o.f[16]) o.f[16][c] = dot * ig2;
        if (o.f[17]) {
            const float plap = (hxp - 2.f * hc + hxm) * rc.fxx + (hyp - 2.f * hc + hym) * rc.fyy +
                               (hzp - 2.f * hc + hzm) * rc.fzz;
            o.f[17][c] = plap * ig2 - dot * lap * (ig2 * ig2);
        }
    }
    return need;
}

// One node of the plain FP64 toolbox (set_calculus_toolbox.cu:9-107), the reference's
// expressions in its order.
template <class Get>
__device__ __forceinline__ void toolbox_point_f64(Get F, int i, int j, int k, int im, int ip, int jm, int jp,
                                                  int km, int kp, long long c, const ToolboxOut<double> &o,
                                                  const Grid &g, double ds_, double thr2ds, double &area,
                                                  double &vol, int &units)
{
    using T = double;
    bool unit = false;
    auto H = [&](int a, int b, int e) { return vmax(F(a, b, e), T(0)); };
    const T dx = (T)g.dx, dy = (T)g.dy, dz = (T)g.dz, ds = (T)ds_;
    const T fc = F(i, j, k);
    const T fxp = F(i, jp, k), fxm = F(i, jm, k), fyp = F(ip, j, k), fym = F(im, j, k);
    const T fzp = F(i, j, kp), fzm = F(i, j, km);
    T fx = (fxp - fxm) / (2 * dx);
    T fy = (fyp - fym) / (2 * dy);
    T fz = (fzp - fzm) / (2 * dz);
    T gm = vmax(sqrt(fx * fx + fy * fy + fz * fz), T(1e-14));
    T fxx = (fxp - 2 * fc + fxm) / (dx * dx);
    T fyy = (fyp - 2 * fc + fym) / (dy * dy);
    T fzz = (fzp - 2 * fc + fzm) / (dz * dz);
    T fxy = (F(ip, jp, k) + F(im, jm, k) - F(ip, jm, k) - F(im, jp, k)) / (4 * ds * ds);
    T fyz = (F(ip, j, kp) + F(im, j, km) - F(ip, j, km) - F(im, j, kp)) / (4 * ds * ds);
    T fzx = (F(i, jp, kp) + F(i, jm, km) - F(i, jp, km) - F(i, jm, kp)) / (4 * ds * ds);
    T lap = fxx + fyy + fzz;
    T r1 = fxx * fx + fxy * fy + fzx * fz;
    T r2 = fxy * fx + fyy * fy + fyz * fz;
    T r3 = fzx * fx + fyz * fy + fzz * fz;
    T gm2 = gm * gm;
    T mean = -lap / gm + (fx * r1 + fy * r2 + fz * r3) / cube(gm);
    const T gm4 = fourth(gm);
    T hc = vmax(fc, T(0));
    T hxp = H(i, jp, k), hxm = H(i, jm, k), hyp = H(ip, j, k), hym = H(im, j, k);
    T hzp = H(i, j, kp), hzm = H(i, j, km);
    T px = (hxp - hxm) / (2 * dx), py = (hyp - hym) / (2 * dy), pz = (hzp - hzm) / (2 * dz);
    T dot = px * fx + py * fy + pz * fz;
    T pxx = (hxp - 2 * hc + hxm) / (dx * dx);
    T pyy = (hyp - 2 * hc + hym) / (dy * dy);
    T pzz = (hzp - 2 * hc + hzm) / (dz * dz);
    T plap = pxx + pyy + pzz;
    T heav = dot / gm2;
    T delta = plap / gm2 - dot * lap / gm4;
    if (fabs(fc) < thr2ds) area += delta;
    if (fc < thr2ds) {
        // heav == 0 (no positive neighbour) gives a volume term of exactly 1
        if (heav == T(0)) {
            unit = true;
        } else {
            const double v1 = 1 - heav;
            if (v1 == 1.0)
                unit = true;
            else
                vol += v1;
        }
    }
    if (o.f[0]) o.f[0][c] = fx;
    if (o.f[1]) o.f[1][c] = fy;
    if (o.f[2]) o.f[2][c] = fz;
    if (o.f[3]) o.f[3][c] = gm;
    if (o.f[4]) o.f[4][c] = fx / gm;
    if (o.f[5]) o.f[5][c] = fy / gm;
    if (o.f[6]) o.f[6][c] = fz / gm;
    if (o.f[7]) o.f[7][c] = fxx;
    if (o.f[8]) o.f[8][c] = fyy;
    if (o.f[9]) o.f[9][c] = fzz;
    if (o.f[10]) o.f[10][c] = fxy;
    if (o.f[11]) o.f[11][c] = fyz;
    if (o.f[12]) o.f[12][c] = fzx;
    if (o.f[13]) o.f[13][c] = lap;
    if (o.f[14]) o.f[14][c] = mean;
    if (o.f[15]) {
        T q1 = (fyy * fzz - fyz * fyz) * fx + (fzx * fyz - fxy * fzz) * fy + (fxy * fyz - fzx * fyy) * fz;
        T q2 = (fyz * fzx - fxy * fzz) * fx + (fxx * fzz - fzx * fzx) * fy + (fzx * fxy - fxx * fyz) * fz;
        T q3 = (fxy * fyz - fyy * fzx) * fx + (fzx * fxy - fxx * fyz) * fy + (fxx * fyy - fxy * fxy) * fz;
        o.f[15][c] = (fx * q1 + fy * q2 + fz * q3) / gm4;
    }
    if (o.f[16]) o.f[16][c] = heav;
    if (o.f[17]) o.f[17][c] = delta;
    units += unit ? 1 : 0;
}

// One node of the toolbox: F(a, b, e) gives the field at row a, column b, page e (clamped
// coordinates), c the node's offset.  Adds the node's FP64 area and volume terms to area /
// vol and counts a volume term of exactly 1 in units.
template <typename T, class Get>
__device__ __forceinline__ void toolbox_point(Get F, int i, int j, int k, int im, int ip, int jm, int jp, int km,
                                              int kp, long long c, const ToolboxOut<T> &o, const Grid &g,
                                              double ds_, T thr2ds, const Recips &rc, double &area, double &vol,
                                              int &units)
{
    static_assert(std::is_same<T, double>::value, "the mixed form's toolbox is k_toolbox_tiled");
    toolbox_point_f64(F, i, j, k, im, ip, jm, jp, km, kp, c, o, g, ds_, thr2ds, area, vol, units);
}

// thr2ds: 2 Ds as the smallest T not below it, so that x < thr2ds in T is exactly
// (double)x < 2 Ds for every x of type T (the reference's FP64 band tests)
template <typename T>
__global__ void __launch_bounds__(NT) k_toolbox(const T *__restrict__ f, ToolboxOut<T> o, Grid g, double ds_,
                                                T thr2ds, double *__restrict__ partials, Recips rc)
{
    const int i = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int k = blockIdx.z;
    double area = 0.0, vol = 0.0;
    int units = 0;  // volume terms equal to exactly 1
    if (i < g.rows && j < g.cols) {
        const long long c = node_index(g, i, j, k);
        // the clamped neighbour coordinates once; node offsets in 32 bits (grids hold fewer
        // than 2^31 nodes)
        const int im = clampi(i - 1, g.rows), ip = clampi(i + 1, g.rows);
        const int jm = clampi(j - 1, g.cols), jp = clampi(j + 1, g.cols);
        const int km = clampi(k - 1, g.pges), kp = clampi(k + 1, g.pges);
        const unsigned rows = (unsigned)g.rows, plane = (unsigned)g.plane;
        auto F = [&](int a, int b, int e) { return __ldg(f + ((unsigned)e * plane + (unsigned)b * rows + (unsigned)a)); };
        toolbox_point<T>(F, i, j, k, im, ip, jm, jp, km, kp, c, o, g, ds_, thr2ds, rc, area, vol, units);
    }
    if (!partials) return;
    // Volume terms equal to exactly 1 (nodes with no positive neighbour) are counted as
    // integers; only warps holding other terms run the FP64 shuffle tree.  Per block:
    // partial = (double)count + FP64 tree sum of the rest, in a fixed order.
    __shared__ double sa[NW], sv[NW];
    __shared__ int sc[NW];
    const int t = threadIdx.y * BX + threadIdx.x;
    const int ones = __reduce_add_sync(0xffffffffu, units);
    if (__any_sync(0xffffffffu, area != 0.0)) area = warp_sum(area);
    if (__any_sync(0xffffffffu, vol != 0.0)) vol = warp_sum(vol);
    if ((t & 31) == 0) {
        sa[t >> 5] = area;
        sv[t >> 5] = vol;
        sc[t >> 5] = ones;
    }
    __syncthreads();
    if (t == 0) {
        double a = 0.0, v = 0.0;
        int n = 0;
        for (int w = 0; w < NW; ++w) {
            a += sa[w];
            v += sv[w];
            n += sc[w];
        }
        const long long b = block_linear();
        partials[2 * b] = a;
        partials[2 * b + 1] = (double)n + v;
    }
}

// The mixed form's toolbox on 2.5D tiles: a block of BX x BY threads owns a tile of BX rows
// x BY columns and marches kz pages along z; the stencil of page k reads a ring of four
// shared planes (the tile with a one-node halo, clamped at the grid edge when loaded), of
// which pages k-1, k, k+1 are live while page k+2 is fetched into registers during the
// page's arithmetic and stored into the slot of page k-2 at its end.  One barrier per
// page.  Each node is read from memory about once (halo re-reads hit L2), instead of
// nineteen times through L1 as in k_toolbox.  Per thread the FP64 area and volume terms
// of its column are summed page by page, then per block in the fixed order of k_toolbox:
// the same terms as k_toolbox, summed in another fixed order.
constexpr int TB_RING = 4;
constexpr int TB_SW = BX + 2, TB_SH = BY + 2, TB_PLANE = TB_SW * TB_SH;

template <typename T>
__global__ void __launch_bounds__(NT, 4) k_toolbox_tiled(const T *__restrict__ f, ToolboxOut<T> o, Grid g, double ds_,
                                                      T thr2ds, double *__restrict__ partials, Recips rc, int kz)
{
    __shared__ T sm[TB_RING][TB_PLANE];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
    const int i0 = blockIdx.x * BX, j0 = blockIdx.y * BY;
    const int i = i0 + tx, j = j0 + ty;
    const int k0 = blockIdx.z * kz, k1 = min(k0 + kz, g.pges);
    const bool active = i < g.rows && j < g.cols;
    const unsigned rows = (unsigned)g.rows, plane = (unsigned)g.plane;
    // this thread's (at most two) elements of a tile plane: in-page offsets of the clamped nodes
    static_assert(TB_PLANE <= 2 * NT, "a tile plane is two elements per thread at most");
    const bool second = tid + NT < TB_PLANE;
    auto in_page = [&](int e) {
        const int sy = e / TB_SW, sx = e - sy * TB_SW;
        return (unsigned)clampi(j0 + sy - 1, g.cols) * rows + (unsigned)clampi(i0 + sx - 1, g.rows);
    };
    const unsigned off0 = in_page(tid), off1 = second ? in_page(tid + NT) : 0u;
    T pre0 = T(0), pre1 = T(0);
    auto fetch = [&](int p) {
        const T *src = f + (unsigned)clampi(p, g.pges) * plane;
        pre0 = __ldg(src + off0);
        if (second) pre1 = __ldg(src + off1);
    };
    auto store = [&](int p) {
        T *dst = sm[p & (TB_RING - 1)];
        dst[tid] = pre0;
        if (second) dst[tid + NT] = pre1;
    };
    for (int p = k0 - 1; p <= k0 + 1; ++p) {
        fetch(p);
        store(p);
    }
    // the clamped neighbour coordinates of the column; a page e (clamped) sits in slot e & 3,
    // which holds plane e while pages e-1 .. e+1 are live
    const int im = clampi(i - 1, g.rows), ip = clampi(i + 1, g.rows);
    const int jm = clampi(j - 1, g.cols), jp = clampi(j + 1, g.cols);
    auto F = [&](int a, int b, int e) { return sm[e & (TB_RING - 1)][(b - j0 + 1) * TB_SW + (a - i0 + 1)]; };
    double area = 0.0, vol = 0.0;
    int units = 0;
    const long long col = (long long)clampi(j, g.cols) * g.rows + clampi(i, g.rows);
    // Per warp, the band nodes waiting for their FP64 area and volume terms (their eight
    // inputs, one column per node), evaluated 32 at a time, one node per lane: a warp with
    // one band node would otherwise issue the FP64 block (1/64 of the FP32 rate on this
    // GPU) for all its lanes.  The queue's order (page, then lane) and each lane's sum are
    // fixed, so the sums stay reproducible.
    __shared__ float q64[NW][8][64];
    float(*Q)[64] = q64[tid >> 5];
    const unsigned lane = tid & 31;
    int qn = 0;  // queued nodes of this warp (warp-uniform)
    auto evaluate = [&](int n) {  // the first n <= 32 queued nodes, lane l the l-th
        if ((int)lane < n) {
            float v[8];
#pragma unroll
            for (int m = 0; m < 8; ++m) v[m] = Q[m][lane];
            band_terms_f64(v, rc, area, vol, units);
        }
    };
    for (int k = k0; k < k1; ++k) {
        // plane k+1 is stored, and no warp reads the slot of page k-2 any more
        __syncthreads();
        fetch(k + 2);
        bool need = false;
        float v[8];
        if (active) {
            const int km = clampi(k - 1, g.pges), kp = clampi(k + 1, g.pges);
            need = toolbox_point_f32(F, i, j, k, im, ip, jm, jp, km, kp, col + (long long)k * g.plane, o, thr2ds, rc, v,
                                     units);
        }
        if (partials) {
            const unsigned m = __ballot_sync(0xffffffffu, need);
            if (m) {
                if (need) {
                    const int r = qn + __popc(m & ((1u << lane) - 1u));
#pragma unroll
                    for (int e = 0; e < 8; ++e) Q[e][r] = v[e];
                }
                qn += __popc(m);
                __syncwarp();
                if (qn >= 32) {
                    evaluate(32);
                    __syncwarp();
                    if ((int)lane < qn - 32) {
#pragma unroll
                        for (int e = 0; e < 8; ++e) Q[e][lane] = Q[e][lane + 32];
                    }
                    __syncwarp();
                    qn -= 32;
                }
            }
        }
        store(k + 2);
    }
    if (!partials) return;
    if (qn > 0) evaluate(qn);
    __shared__ double sa[NW], sv[NW];
    __shared__ int sc[NW];
    const int ones = __reduce_add_sync(0xffffffffu, units);
    if (__any_sync(0xffffffffu, area != 0.0)) area = warp_sum(area);
    if (__any_sync(0xffffffffu, vol != 0.0)) vol = warp_sum(vol);
    if ((tid & 31) == 0) {
        sa[tid >> 5] = area;
        sv[tid >> 5] = vol;
        sc[tid >> 5] = ones;
    }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, v = 0.0;
        int n = 0;
        for (int w = 0; w < NW; ++w) {
            a += sa[w];
            v += sv[w];
            n += sc[w];
        }
        const long long b = block_linear();
        partials[2 * b] = a;
        partials[2 * b + 1] = (double)n + v;
    }
}

// per-block max |f| over the band |phi| < band (p00_test_singlephase_relax.m:86-89)
// In T: the band test against `band` rounded up to T (exactly the FP64 test) and the
// maximum of |f| (exact: conversion to double is monotonic), converted once per block.
template <typename T>
__global__ void __launch_bounds__(NT) k_band_maxabs(const T *__restrict__ f, const T *__restrict__ phi, T band,
                                                    Grid g, double *__restrict__ partials)
{
    const int i = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int k = blockIdx.z;
    T m = T(0);
    if (i < g.rows && j < g.cols) {
        const long long c = node_index(g, i, j, k);
        if (fabs(__ldg(phi + c)) < band) m = fabs(__ldg(f + c));
    }
    __shared__ T s[NW];
    const int t = threadIdx.y * BX + threadIdx.x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((t & 31) == 0) s[t >> 5] = m;
    __syncthreads();
    if (t == 0) {
        T r = T(0);
        for (int w = 0; w < NW; ++w) r = fmax(r, s[w]);
        partials[block_linear()] = (double)r;
    }
}

// the smallest T not below x: x < round_up<T>(x') in T  <=>  (double)x < x'
template <typename T> T round_up(double x);
template <> double round_up<double>(double x) { return x; }
template <> float round_up<float>(double x)
{
    float r = (float)x;
    if ((double)r < x) r = std::nextafter(r, std::numeric_limits<float>::infinity());
    return r;
}

}  // namespace

template <typename T>
cudaError_t launch_toolbox(const T *phi, ToolboxOut<T> out, const Grid &g, double ds, double *partials,
                           int *nblocks, cudaStream_t s)
{
    const double ds2 = ds * ds;
    const Recips rc{1 / (2 * g.dx),
                    1 / (2 * g.dy),
                    1 / (2 * g.dz),
                    1 / (g.dx * g.dx),
                    1 / (g.dy * g.dy),
                    1 / (g.dz * g.dz),
                    (float)(1 / (2 * g.dx)),
                    (float)(1 / (2 * g.dy)),
                    (float)(1 / (2 * g.dz)),
                    (float)(1 / (g.dx * g.dx)),
                    (float)(1 / (g.dy * g.dy)),
                    (float)(1 / (g.dz * g.dz)),
                    (float)(1 / (4 * ds2))};
    if constexpr (std::is_same<T, float>::value) {
        // pages per block: a function of the grid alone (the partials, and so the sums, do
        // not depend on the device), about 2400 blocks where the grid allows, 16 pages at most
        dim3 gr = node_grid(g);
        const long long tiles = (long long)gr.x * gr.y;
        const int kz = (int)std::min<long long>(16, std::max<long long>(1, tiles * g.pges / 2400));
        gr.z = (unsigned)((g.pges + kz - 1) / kz);
        if (nblocks) *nblocks = (int)(tiles * gr.z);
        k_toolbox_tiled<T><<<gr, dim3(BX, BY), 0, s>>>(phi, out, g, ds, round_up<T>(2 * ds), partials, rc, kz);
    } else {
        // the plain form: one node per thread, the reference's summation blocks
        if (nblocks) *nblocks = toolbox_partial_blocks(g);
        k_toolbox<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi, out, g, ds, round_up<T>(2 * ds), partials, rc);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_band_maxabs(const T *f, const T *phi, double band, const Grid &g, double *partials,
                               int *nblocks, cudaStream_t s)
{
    if (nblocks) *nblocks = toolbox_partial_blocks(g);
    k_band_maxabs<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(f, phi, round_up<T>(band), g, partials);
    return cudaGetLastError();
}

}  // namespace vsl
