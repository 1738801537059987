// vsl_auxi.cuh -- the calculus toolbox of the auxiliary level set A that marks the
// domains of a multiphase vesicle on the surface F = 0 (auxi_set_calculus_toolbox.cu:10-199,
// GPUAsetCalculusToolBox.m:2-63) and the masked FP64 surface and line integrals of
// SDF3.m:82-85, 212-227.  Templated on the field type; included by vsl_auxi_f64.cu (no
// multiply-add contraction, the reference's rounding) and vsl_auxi_f32.cu (mixed form).
//
// The fused form reads only A and F: F's gradient, Hessian, normal and Heaviside are
// recomputed from F's stencil with the calculus toolbox's own expressions instead of
// being read back from 14 stored toolbox fields.  Pass 1 writes the requested fields of
// the kernel plus the Heaviside functions of A and F; pass 2 forms AFDiracDelta and
// ADiracDeltaDn with SD.GD3's periodic operators, as the MATLAB method does.
#pragma once

#include <cmath>
#include <limits>

#include "vsl_internal.h"

namespace vsl {
namespace {

constexpr int ANT = BX * BY;
constexpr int ANW = ANT / 32;

template <typename T> __device__ __forceinline__ T a_sq(T x) { return x * x; }
template <typename T> __device__ __forceinline__ T a_cube(T x);
template <> __device__ __forceinline__ double a_cube<double>(double x) { return pow_cr<3>(x); }
template <> __device__ __forceinline__ float a_cube<float>(float x) { return x * x * x; }
template <typename T> __device__ __forceinline__ T a_fourth(T x);
template <> __device__ __forceinline__ double a_fourth<double>(double x) { return pow_cr<4>(x); }
template <> __device__ __forceinline__ float a_fourth<float>(float x) { return (x * x) * (x * x); }

// the vector norm of shared_utilities.cup:8-12, floored at 1e-14
template <typename T> __device__ __forceinline__ T a_norm(T x, T y, T z) { return vmax(sqrt(x * x + y * y + z * z), T(1e-14)); }

__device__ __forceinline__ bool a_node(const Grid &g, int &i, int &j, int &k, long long &c)
{
    i = blockIdx.x * BX + threadIdx.x;
    j = blockIdx.y * BY + threadIdx.y;
    k = blockIdx.z;
    if (i >= g.rows || j >= g.cols) return false;
    c = node_index(g, i, j, k);
    return true;
}

// F's toolbox values at one node: gradient, |grad F| (floored), Hessian, normal, and the
// Heaviside function from the primal max(F, 0) -- k_toolbox's expressions in its order
template <typename T> struct FPart {
    T fx, fy, fz, gm, nx, ny, nz, fxx, fyy, fzz, fxy, fyz, fzx, heav;
};
template <typename T>
__device__ __forceinline__ FPart<T> f_part(const T *__restrict__ f, const Grid &g, int i, int j, int k, long long c,
                                           T dx, T dy, T dz, T ds)
{
    auto F = [&](int a, int b, int e) { return __ldg(f + clamped_index(g, a, b, e)); };
    FPart<T> r;
    const T fc = __ldg(f + c);
    const T fxp = F(i, j + 1, k), fxm = F(i, j - 1, k), fyp = F(i + 1, j, k), fym = F(i - 1, j, k);
    const T fzp = F(i, j, k + 1), fzm = F(i, j, k - 1);
    r.fx = (fxp - fxm) / (2 * dx);
    r.fy = (fyp - fym) / (2 * dy);
    r.fz = (fzp - fzm) / (2 * dz);
    r.gm = vmax(sqrt(r.fx * r.fx + r.fy * r.fy + r.fz * r.fz), T(1e-14));
    r.nx = r.fx / r.gm;
    r.ny = r.fy / r.gm;
    r.nz = r.fz / r.gm;
    r.fxx = (fxp - 2 * fc + fxm) / (dx * dx);
    r.fyy = (fyp - 2 * fc + fym) / (dy * dy);
    r.fzz = (fzp - 2 * fc + fzm) / (dz * dz);
    r.fxy = (F(i + 1, j + 1, k) + F(i - 1, j - 1, k) - F(i + 1, j - 1, k) - F(i - 1, j + 1, k)) / (4 * ds * ds);
    r.fyz = (F(i + 1, j, k + 1) + F(i - 1, j, k - 1) - F(i + 1, j, k - 1) - F(i - 1, j, k + 1)) / (4 * ds * ds);
    r.fzx = (F(i, j + 1, k + 1) + F(i, j - 1, k - 1) - F(i, j + 1, k - 1) - F(i, j - 1, k + 1)) / (4 * ds * ds);
    const T px = (vmax(fxp, T(0)) - vmax(fxm, T(0))) / (2 * dx);
    const T py = (vmax(fyp, T(0)) - vmax(fym, T(0))) / (2 * dy);
    const T pz = (vmax(fzp, T(0)) - vmax(fzm, T(0))) / (2 * dz);
    r.heav = (px * r.fx + py * r.fy + pz * r.fz) / (r.gm * r.gm);
    return r;
}

// The 27 fields of auxi_set_calculus_toolbox at one node, in the kernel's argument order
enum AuxField {
    AU_AX, AU_AY, AU_AZ, AU_AGRADMAG, AU_CX, AU_CY, AU_CZ, AU_NORMCROSS, AU_TX, AU_TY, AU_TZ, AU_NX, AU_NY, AU_NZ,
    AU_AXX, AU_AYY, AU_AZZ, AU_AXY, AU_AYZ, AU_AZX, AU_ALAP, AU_GEODESIC, AU_NORMALCURV, AU_TORSION, AU_BPERP,
    AU_AHEAV, AU_ADELTA, AU_KERNEL_FIELDS
};

// auxi_set_calculus_toolbox.cu:27-197 at node (i,j,k): A's central differences (clamped,
// `Aat`), the primal of its Heaviside (`Pat`), F's values at the node given.
template <typename T, class AFn, class PFn>
__device__ __forceinline__ void aux_core(AFn Aat, PFn Pat, const FPart<T> &fp, int i, int j, int k, T dx, T dy, T dz,
                                         T ds, T v[AU_KERNEL_FIELDS])
{
    const T ac = Aat(i, j, k);
    const T axp = Aat(i, j + 1, k), axm = Aat(i, j - 1, k), ayp = Aat(i + 1, j, k), aym = Aat(i - 1, j, k);
    const T azp = Aat(i, j, k + 1), azm = Aat(i, j, k - 1);
    const T ax = (axp - axm) / (2 * dx);
    const T ay = (ayp - aym) / (2 * dy);
    const T az = (azp - azm) / (2 * dz);
    const T agm = a_norm(ax, ay, az);
    v[AU_AX] = ax;
    v[AU_AY] = ay;
    v[AU_AZ] = az;
    v[AU_AGRADMAG] = agm;
    const T fx = fp.fx, fy = fp.fy, fz = fp.fz;
    const T cx = fy * az - fz * ay, cy = fz * ax - fx * az, cz = fx * ay - fy * ax;
    const T ncr = a_norm(cx, cy, cz);
    v[AU_CX] = cx;
    v[AU_CY] = cy;
    v[AU_CZ] = cz;
    v[AU_NORMCROSS] = ncr;
    const T tx = cx / ncr, ty = cy / ncr, tz = cz / ncr;
    v[AU_TX] = tx;
    v[AU_TY] = ty;
    v[AU_TZ] = tz;
    const T nx = ty * fp.nz - tz * fp.ny, ny = tz * fp.nx - tx * fp.nz, nz = tx * fp.ny - ty * fp.nx;
    v[AU_NX] = nx;
    v[AU_NY] = ny;
    v[AU_NZ] = nz;
    const T axx = (axp - 2 * ac + axm) / (dx * dx);
    const T ayy = (ayp - 2 * ac + aym) / (dy * dy);
    const T azz = (azp - 2 * ac + azm) / (dz * dz);
    const T axy = (Aat(i + 1, j + 1, k) + Aat(i - 1, j - 1, k) - Aat(i + 1, j - 1, k) - Aat(i - 1, j + 1, k)) / (4 * ds * ds);
    const T ayz = (Aat(i + 1, j, k + 1) + Aat(i - 1, j, k - 1) - Aat(i + 1, j, k - 1) - Aat(i - 1, j, k + 1)) / (4 * ds * ds);
    const T azx = (Aat(i, j + 1, k + 1) + Aat(i, j - 1, k - 1) - Aat(i, j + 1, k - 1) - Aat(i, j - 1, k + 1)) / (4 * ds * ds);
    const T alap = axx + ayy + azz;
    v[AU_AXX] = axx;
    v[AU_AYY] = ayy;
    v[AU_AZZ] = azz;
    v[AU_AXY] = axy;
    v[AU_AYZ] = ayz;
    v[AU_AZX] = azx;
    v[AU_ALAP] = alap;
    const T fxx = fp.fxx, fyy = fp.fyy, fzz = fp.fzz, fxy = fp.fxy, fyz = fp.fyz, fzx = fp.fzx, fgm = fp.gm;
    // geodesic curvature n . ((H_F t) x grad A + grad F x (H_A t)) / |grad F x grad A|
    T vx = tx * fxx + ty * fxy + tz * fzx;
    T vy = tx * fxy + ty * fyy + tz * fyz;
    T vz = tx * fzx + ty * fyz + tz * fzz;
    const T w1x = vy * az - vz * ay, w1y = vz * ax - vx * az, w1z = vx * ay - vy * ax;
    vx = tx * axx + ty * axy + tz * azx;
    vy = tx * axy + ty * ayy + tz * ayz;
    vz = tx * azx + ty * ayz + tz * azz;
    const T w2x = fy * vz - fz * vy, w2y = fz * vx - fx * vz, w2z = fx * vy - fy * vx;
    v[AU_GEODESIC] = (nx * (w1x + w2x) + ny * (w1y + w2y) + nz * (w1z + w2z)) / ncr;
    // grad N = H_F / |grad F| - grad F (H_F grad F)^T / |grad F|^3
    const T g3 = a_cube(fgm);
    const T r1 = fxx * fx + fxy * fy + fzx * fz;
    const T r2 = fxy * fx + fyy * fy + fyz * fz;
    const T r3 = fzx * fx + fyz * fy + fzz * fz;
    const T Nxx = fxx / fgm - fx * r1 / g3, Nyx = fxy / fgm - fy * r1 / g3, Nzx = fzx / fgm - fz * r1 / g3;
    const T Nxy = fxy / fgm - fx * r2 / g3, Nyy = fyy / fgm - fy * r2 / g3, Nzy = fyz / fgm - fz * r2 / g3;
    const T Nxz = fzx / fgm - fx * r3 / g3, Nyz = fyz / fgm - fy * r3 / g3, Nzz = fzz / fgm - fz * r3 / g3;
    vx = Nxx * tx + Nxy * ty + Nxz * tz;
    vy = Nyx * tx + Nyy * ty + Nyz * tz;
    vz = Nzx * tx + Nzy * ty + Nzz * tz;
    v[AU_NORMALCURV] = -(tx * vx + ty * vy + tz * vz);
    vx = Nxx * nx + Nxy * ny + Nxz * nz;
    vy = Nyx * nx + Nyy * ny + Nyz * nz;
    vz = Nzx * nx + Nzy * ny + Nzz * nz;
    v[AU_TORSION] = -(tx * vx + ty * vy + tz * vz);
    v[AU_BPERP] = -(nx * vx + ny * vy + nz * vz);
    // Heaviside and Dirac functions of A from its primal
    const T pc = Pat(i, j, k);
    const T pxp = Pat(i, j + 1, k), pxm = Pat(i, j - 1, k), pyp = Pat(i + 1, j, k), pym = Pat(i - 1, j, k);
    const T pzp = Pat(i, j, k + 1), pzm = Pat(i, j, k - 1);
    const T px = (pxp - pxm) / (2 * dx), py = (pyp - pym) / (2 * dy), pz = (pzp - pzm) / (2 * dz);
    const T dot = px * ax + py * ay + pz * az;
    v[AU_AHEAV] = dot / a_sq(agm);
    const T pxx = (pxp - 2 * pc + pxm) / (dx * dx);
    const T pyy = (pyp - 2 * pc + pym) / (dy * dy);
    const T pzz = (pzp - 2 * pc + pzm) / (dz * dz);
    const T plap = pxx + pyy + pzz;
    v[AU_ADELTA] = plap / a_sq(agm) - dot * alap / a_fourth(agm);
}

// the reference kernel's own form: F's toolbox fields and AHPrimal read from arrays
template <typename T>
__global__ void __launch_bounds__(ANT) k_auxi_dropin(AuxOut<T> o, const T *__restrict__ lsf,
                                                     const T *__restrict__ ahp, AuxFIn<T> fin, Grid g, T ds)
{
    int i, j, k;
    long long c;
    if (!a_node(g, i, j, k, c)) return;
    const T dx = (T)g.dx, dy = (T)g.dy, dz = (T)g.dz;
    FPart<T> fp;
    fp.fx = fin.f[0][c];
    fp.fy = fin.f[1][c];
    fp.fz = fin.f[2][c];
    fp.gm = fin.f[3][c];
    fp.nx = fin.f[4][c];
    fp.ny = fin.f[5][c];
    fp.nz = fin.f[6][c];
    fp.fxx = fin.f[7][c];
    fp.fyy = fin.f[8][c];
    fp.fzz = fin.f[9][c];
    fp.fxy = fin.f[10][c];
    fp.fyz = fin.f[11][c];
    fp.fzx = fin.f[12][c];
    T v[AU_KERNEL_FIELDS];
    aux_core<T>([&](int a, int b, int e) { return __ldg(lsf + clamped_index(g, a, b, e)); },
                [&](int a, int b, int e) { return __ldg(ahp + clamped_index(g, a, b, e)); }, fp, i, j, k, dx, dy, dz,
                ds, v);
#pragma unroll
    for (int q = 0; q < AU_KERNEL_FIELDS; ++q) o.f[q][c] = v[q];
}

// pass 1 of the fused form: F recomputed, AHPrimal = max(A, 0) on the fly; writes the
// requested fields, and the values pass 2 needs into `keep` (outputs or workspace):
// C, |C|, |grad A|, ADiracDelta, AHeaviside and F's Heaviside
template <typename T>
__global__ void __launch_bounds__(ANT) k_aux_pass1(const T *__restrict__ A, const T *__restrict__ F, AuxOut<T> o,
                                                   AuxKeep<T> keep, Grid g, T ds)
{
    int i, j, k;
    long long c;
    if (!a_node(g, i, j, k, c)) return;
    const T dx = (T)g.dx, dy = (T)g.dy, dz = (T)g.dz;
    const FPart<T> fp = f_part(F, g, i, j, k, c, dx, dy, dz, ds);
    T v[AU_KERNEL_FIELDS];
    aux_core<T>([&](int a, int b, int e) { return __ldg(A + clamped_index(g, a, b, e)); },
                [&](int a, int b, int e) { return vmax(__ldg(A + clamped_index(g, a, b, e)), T(0)); }, fp, i, j, k,
                dx, dy, dz, ds, v);
#pragma unroll
    for (int q = 0; q < AU_KERNEL_FIELDS; ++q)
        if (o.f[q]) o.f[q][c] = v[q];
    keep.cx[c] = v[AU_CX];
    keep.cy[c] = v[AU_CY];
    keep.cz[c] = v[AU_CZ];
    keep.ncr[c] = v[AU_NORMCROSS];
    keep.agm[c] = v[AU_AGRADMAG];
    keep.adelta[c] = v[AU_ADELTA];
    keep.aheav[c] = v[AU_AHEAV];
    keep.fheav[c] = fp.heav;
}

// periodic neighbours of SD.GD3 (circshift)
struct PNb {
    int ip, im, jp, jm, kp, km;
};
__device__ __forceinline__ PNb periodic_nb(const Grid &g, int i, int j, int k)
{
    PNb n;
    n.jp = j + 1 == g.cols ? 0 : j + 1;
    n.jm = j == 0 ? g.cols - 1 : j - 1;
    n.ip = i + 1 == g.rows ? 0 : i + 1;
    n.im = i == 0 ? g.rows - 1 : i - 1;
    n.kp = k + 1 == g.pges ? 0 : k + 1;
    n.km = k == 0 ? g.pges - 1 : k - 1;
    return n;
}

// pass 2: AFDiracDelta = (C . (grad H_F x grad H_A)) / |C|^2 with GD3.Gradient, and
// ADiracDeltaDn = (Laplacian(H_A) - ADiracDelta Laplacian(A)) / |grad A| with GD3.Laplacian
// (GPUAsetCalculusToolBox.m:56-61)
template <typename T>
__global__ void __launch_bounds__(ANT) k_aux_pass2(const T *__restrict__ A, AuxKeepC<T> keep, T *__restrict__ afd,
                                                   T *__restrict__ addn, Grid g)
{
    int i, j, k;
    long long c;
    if (!a_node(g, i, j, k, c)) return;
    const T dx = (T)g.dx, dy = (T)g.dy, dz = (T)g.dz;
    const PNb n = periodic_nb(g, i, j, k);
    auto at = [&](const T *f, int a, int b, int e) { return __ldg(f + node_index(g, a, b, e)); };
    if (afd) {
        const T *h1 = keep.aheav, *h2 = keep.fheav;
        const T h1x = (at(h1, i, n.jp, k) - at(h1, i, n.jm, k)) / (2 * dx);
        const T h1y = (at(h1, n.ip, j, k) - at(h1, n.im, j, k)) / (2 * dy);
        const T h1z = (at(h1, i, j, n.kp) - at(h1, i, j, n.km)) / (2 * dz);
        const T h2x = (at(h2, i, n.jp, k) - at(h2, i, n.jm, k)) / (2 * dx);
        const T h2y = (at(h2, n.ip, j, k) - at(h2, n.im, j, k)) / (2 * dy);
        const T h2z = (at(h2, i, j, n.kp) - at(h2, i, j, n.km)) / (2 * dz);
        const T chx = h2y * h1z - h2z * h1y, chy = h2z * h1x - h2x * h1z, chz = h2x * h1y - h2y * h1x;
        const T dot = __ldg(keep.cx + c) * chx + __ldg(keep.cy + c) * chy + __ldg(keep.cz + c) * chz;
        const T ncr = __ldg(keep.ncr + c);
        afd[c] = dot / (ncr * ncr);
    }
    if (addn) {
        auto lap = [&](const T *f) {
            const T fc = __ldg(f + c);
            const T fxx = (at(f, i, n.jp, k) - T(2) * fc + at(f, i, n.jm, k)) / (dx * dx);
            const T fyy = (at(f, n.ip, j, k) - T(2) * fc + at(f, n.im, j, k)) / (dy * dy);
            const T fzz = (at(f, i, j, n.kp) - T(2) * fc + at(f, i, j, n.km)) / (dz * dz);
            return fxx + fyy + fzz;
        };
        addn[c] = (lap(keep.aheav) - __ldg(keep.adelta + c) * lap(A)) / __ldg(keep.agm + c);
    }
}

// Masked FP64 integral (SDF3.m:82-85, 212-227): sum over |F| < 2Ds (and |A| < 2Ds where A
// is given) of ((f0 * f1) * f2) * (1 - om), absent factors skipped (an absent f0 is 1),
// the products in FP64 in MATLAB's left-to-right order; per-block partials in a fixed order.
template <typename T>
__global__ void __launch_bounds__(ANT) k_masked_sum(const T *__restrict__ F, const T *__restrict__ A,
                                                    const T *__restrict__ f0, const T *__restrict__ f1,
                                                    const T *__restrict__ f2, const T *__restrict__ om, T thr,
                                                    Grid g, double *__restrict__ partials)
{
    int i, j, k;
    long long c = 0;
    double v = 0.0;
    if (a_node(g, i, j, k, c) && fabs(__ldg(F + c)) < thr && (!A || fabs(__ldg(A + c)) < thr)) {
        v = f0 ? (double)__ldg(f0 + c) : 1.0;
        if (f1) v *= (double)__ldg(f1 + c);
        if (f2) v *= (double)__ldg(f2 + c);
        if (om) v *= 1.0 - (double)__ldg(om + c);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __shared__ double s[ANW];
    const int t = threadIdx.y * BX + threadIdx.x;
    if ((t & 31) == 0) s[t >> 5] = v;
    __syncthreads();
    if (t == 0) {
        double r = 0.0;
        for (int w = 0; w < ANW; ++w) r += s[w];
        partials[blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z)] = r;
    }
}

// the smallest T not below x: x < a_round_up<T>(x') in T  <=>  (double)x < x'
template <typename T> T a_round_up(double x);
template <> double a_round_up<double>(double x) { return x; }
template <> float a_round_up<float>(double x)
{
    float r = (float)x;
    if ((double)r < x) r = std::nextafter(r, std::numeric_limits<float>::infinity());
    return r;
}

}  // namespace

template <typename T>
cudaError_t launch_aux_toolbox(const T *A, const T *F, AuxOut<T> o, AuxKeep<T> keep, const Grid &g, double ds,
                               cudaStream_t s)
{
    const dim3 gr = node_grid(g), bl(BX, BY);
    k_aux_pass1<T><<<gr, bl, 0, s>>>(A, F, o, keep, g, (T)ds);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    T *afd = o.f[AU_KERNEL_FIELDS], *addn = o.f[AU_KERNEL_FIELDS + 1];
    if (!afd && !addn) return cudaSuccess;
    AuxKeepC<T> kc{keep.cx, keep.cy, keep.cz, keep.ncr, keep.agm, keep.adelta, keep.aheav, keep.fheav};
    k_aux_pass2<T><<<gr, bl, 0, s>>>(A, kc, afd, addn, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_masked_sum(const T *F, const T *A, const T *f0, const T *f1, const T *f2, const T *om,
                              const Grid &g, double ds, double *partials, int *nblocks, cudaStream_t s)
{
    if (nblocks) *nblocks = toolbox_partial_blocks(g);
    k_masked_sum<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(F, A, f0, f1, f2, om, a_round_up<T>(2 * ds), g, partials);
    return cudaGetLastError();
}

#define VSL_INSTANTIATE_AUXI(T)                                                                                     \
    template cudaError_t launch_aux_toolbox<T>(const T *, const T *, AuxOut<T>, AuxKeep<T>, const Grid &, double,   \
                                               cudaStream_t);                                                       \
    template cudaError_t launch_masked_sum<T>(const T *, const T *, const T *, const T *, const T *, const T *,     \
                                              const Grid &, double, double *, int *, cudaStream_t);

}  // namespace vsl
