// vsl_adjoint.cu -- reverse-mode (adjoint) kernels of the WENO5 TVD-RK3 advection and
// reinitialization stages, and of the sub-cell distances the reinitialization reads.
//
// A fused stage writes  out = a * phi_n + b * (phi_s - step(phi_s)).  Its adjoint, given
// lam = dL/d out, is
//     dL/d phi_s = b * lam - J^T (b * lam),   dL/d phi_n += a * lam,
// with J the Jacobian of `step`.  Row c of J touches the 7 values of each axis line
// through c (clamped at the grid edge), so J^T is applied in two deterministic passes:
//   1. per node c, the local partials d step_c / d p_ax[o] (o = 0..6 along axis ax) are
//      evaluated by running the forward per-node code on dual numbers, scaled by
//      b * lam_c and stored in 21 slots W[ax*7 + o][c] (slot-major, coalesced);
//   2. per node j, every (c, ax, o) whose clamped stencil position is j is summed in a
//      fixed order (no atomics), giving (J^T b lam)_j.
// Partials with respect to the other inputs of a stage (the velocity of advection, the
// six interface distances of reinitialization) are accumulated per node in the same
// pass.  The distance adjoints are carried back to the field the distances were computed
// from by the implicit-function derivative of each root (k_adj_dist_edges).
//
// Every update is differentiated exactly as evaluated: WENO weights including their
// epsilon, the upwind and Godunov switches, the interface insertion and the minimum over
// the six distances in the pseudo-time step.  At a switch, the branch taken is
// differentiated.  The mask (sign of the field when a reinitialization starts) and the
// fixed-node test are piecewise constant and carry no derivative.
#include <cmath>

#include "vsl_dual.cuh"
#include "vsl_internal.h"

namespace vsl {
namespace {

// classification byte of the fused kernels: bit 6 mask (phi < 0 at the start), bit 7
// fixed node (a distance below 1e-6 dx)
constexpr uint8_t CLS_MASK = 0x40;
constexpr uint8_t CLS_FIXED = 0x80;
constexpr int SLOTS = 21;

__device__ __forceinline__ bool adj_node(const Grid &g, int &i, int &j, int &k, long long &c)
{
    i = blockIdx.x * BX + threadIdx.x;
    j = blockIdx.y * BY + threadIdx.y;
    k = blockIdx.z;
    if (i >= g.rows || j >= g.cols) return false;
    c = node_index(g, i, j, k);
    return true;
}

__device__ __forceinline__ void adj_node_of(const Grid &g, long long c, int &i, int &j, int &k)
{
    k = (int)(c / g.plane);
    const long long r = c - (long long)k * g.plane;
    j = (int)(r / g.rows);
    i = (int)(r - (long long)j * g.rows);
}

// Forward/backward derivative pair of one axis line and its partials with respect to
// the seven line values (tangents 0..6) and the two interface distances r1, l1 (7, 8):
// the uniform WENO5 pair, or the nonuniform one with the interface inserted.
template <typename T>
__device__ __forceinline__ void axis_pair_jac(const T p[7], T h, bool iface, T r1, T l1, Dual<T, 9> &f,
                                              Dual<T, 9> &b)
{
    using D = Dual<T, 9>;
    D P[7];
#pragma unroll
    for (int o = 0; o < 7; ++o) P[o] = D::var(p[o], o);
    if (iface)
        interface_pair<D>(P, D::var(r1, 7), D::var(l1, 8), D((double)h), D(0.0), D(0.0), false, f, b);
    else
        weno5_pair_plain<D>(P, D((double)h), f, b);
}

// ---------------------------------------------------------------------------------------
// advection stage: step = dt * sum_ax (min(0, v) D+ + max(0, v) D-)  (uniform WENO5)
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(BX *BY) k_adj_advect_jac(const T *__restrict__ ps, Ptr3<const T> v,
                                                             const double *__restrict__ dt,
                                                             const T *__restrict__ lam, T coef, T *__restrict__ W,
                                                             Ptr3<T> gv, Grid g)
{
    int i, j, k;
    long long c;
    if (!adj_node(g, i, j, k, c)) return;
    const T lc = coef * __ldg(lam + c) * (T)__ldg(dt);
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
        using D = Dual<T, 7>;
        T p[7];
        load_line7(ps, axis_line(g, i, j, k, ax), p);
        D P[7];
#pragma unroll
        for (int o = 0; o < 7; ++o) P[o] = D::var(p[o], o);
        D f, b;
        weno5_pair_plain<D>(P, D(axis_h(g, ax)), f, b);
        const T va = __ldg(v.p[ax] + c);
        const T vm = vmin(T(0), va), vp = vmax(T(0), va);
#pragma unroll
        for (int o = 0; o < 7; ++o) W[(long long)(ax * 7 + o) * g.num + c] = lc * (vm * f.d[o] + vp * b.d[o]);
        // d step / d v: D- where v > 0, D+ otherwise (the branches of max/min above)
        gv.p[ax][c] -= lc * (va > T(0) ? b.v : f.v);
    }
}

// ---------------------------------------------------------------------------------------
// reinitialization stage: step = (|grad|_Godunov - 1) * 0.3 min(dist) * (mask ? -1 : 1)
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(BX *BY) k_adj_reinit_jac(const T *__restrict__ ps, const uint8_t *__restrict__ flags,
                                                             Ptr6<const T> d, const T *__restrict__ lam, T coef,
                                                             T *__restrict__ W, Ptr6<T> mu, Grid g)
{
    int i, j, k;
    long long c;
    if (!adj_node(g, i, j, k, c)) return;
    const uint8_t fl = __ldg(flags + c);
    if (fl & CLS_FIXED) {
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) W[(long long)s * g.num + c] = T(0);
        return;
    }
    const T lc = coef * __ldg(lam + c);
    const T h[3] = {(T)g.dx, (T)g.dy, (T)g.dz};
    // the six distances (stored where flagged, the spacing elsewhere) and the pseudo-time
    // step 0.3 * min, with tangents over the flagged ones
    using D6 = Dual<T, 6>;
    T dist[6];
    D6 dv[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const bool f = fl & (1u << q);
        dist[q] = f ? __ldg(d.p[q] + c) : h[q / 2];
        dv[q] = f ? D6::var(dist[q], q) : D6((double)dist[q]);
    }
    const D6 dtd = T(0.3) * vmin(vmin(dv[0], dv[1]), vmin(vmin(dv[2], dv[3]), vmin(dv[4], dv[5])));
    const bool neg = fl & CLS_MASK;
    const T sgn = neg ? T(-1) : T(1);

    T jf[3][9], jb[3][9];
    D6 x[6];
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
        T p[7];
        load_line7(ps, axis_line(g, i, j, k, ax), p);
        const bool iface = p[2] * p[3] < T(0) || p[3] * p[4] < T(0);
        Dual<T, 9> f, b;
        axis_pair_jac<T>(p, h[ax], iface, dist[2 * ax], dist[2 * ax + 1], f, b);
#pragma unroll
        for (int o = 0; o < 9; ++o) {
            jf[ax][o] = f.d[o];
            jb[ax][o] = b.d[o];
        }
        x[2 * ax] = D6::var(f.v, 2 * ax);
        x[2 * ax + 1] = D6::var(b.v, 2 * ax + 1);
    }
    const D6 G = godunov_norm<D6>(neg, x[0], x[1], x[2], x[3], x[4], x[5]);
    const T s_dt = dtd.v * sgn;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        const T gf = G.d[2 * ax] * s_dt, gb = G.d[2 * ax + 1] * s_dt;
#pragma unroll
        for (int o = 0; o < 7; ++o) W[(long long)(ax * 7 + o) * g.num + c] = lc * (gf * jf[ax][o] + gb * jb[ax][o]);
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        if (!(fl & (1u << q))) continue;
        const int ax = q / 2, slot = 7 + (q & 1);
        const T ds = G.d[2 * ax] * s_dt * jf[ax][slot] + G.d[2 * ax + 1] * s_dt * jb[ax][slot] +
                     (G.v - T(1)) * sgn * dtd.d[q];
        mu.p[q][c] -= lc * ds;
    }
}

// ---------------------------------------------------------------------------------------
// transpose pass: out_j = alpha * lam_j - sum of W over the stencil positions equal to j
// (+ acc_j)
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(BX *BY) k_adj_gather(const T *__restrict__ W, const T *lam, T alpha,
                                                         const T *__restrict__ acc, T *out, Grid g)
{
    int i, j, k;
    long long c;
    if (!adj_node(g, i, j, k, c)) return;
    T s = T(0);
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
        const AxisLine L = axis_line(g, i, j, k, ax);
        const T *Wa = W + (long long)(ax * 7) * g.num + L.base;
        const int cj = L.c, n = L.n;
        s += Wa[3 * g.num + (long long)cj * L.stride];
        // sources whose offset o lands exactly on cj
#pragma unroll
        for (int o = 0; o < 7; ++o) {
            if (o == 3) continue;
            const int ci = cj - (o - 3);
            if (ci >= 0 && ci < n) s += Wa[(long long)o * g.num + (long long)ci * L.stride];
        }
        // sources whose offset ran past an edge and was clamped onto cj
        if (cj == 0) {
            for (int ci = 0; ci < min(3, n); ++ci)
                for (int o = 0; o <= 2 - ci; ++o) s += Wa[(long long)o * g.num + (long long)ci * L.stride];
        }
        if (cj == n - 1) {
            for (int ci = max(0, n - 3); ci < n; ++ci)
                for (int o = n + 3 - ci; o <= 6; ++o) s += Wa[(long long)o * g.num + (long long)ci * L.stride];
        }
    }
    const T a = acc ? acc[c] : T(0);
    out[c] = alpha * lam[c] - s + a;
}

// acc = (init ? 0 : acc) + a * lam
template <typename T>
__global__ void k_adj_axpy(T *acc, const T *__restrict__ lam, T a, bool init, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        acc[t] = (init ? T(0) : acc[t]) + a * lam[t];
}

// ---------------------------------------------------------------------------------------
// distances: d/dv of the root of each crossed edge
// ---------------------------------------------------------------------------------------

// the quadratic ENO distance next to a kink, on dual numbers (same formula as the double
// eno2_distance)
template <typename D> __device__ D eno2_distance_dual(D a, D b, D c, D d, double h)
{
    const double eps = 10e-10;
    const D d2 = minmod(c - 2.0 * b + a, d - 2.0 * c + b);
    if (d2 > D(eps) || d2 < D(-eps)) {
        const D disc = sqr(0.5 * d2 - b - c) - 4. * b * c;
        return h * (D(0.5) + (b - c - sgn1((b - c).v) * sqrt(disc)) / d2);
    }
    return h * b / (b - c);
}

// jd[s] = d dist / d v[s] of quintic_distance(v, h): the implicit-function derivative
// -L_s(t) / P'(t) of the fitted root t (zero where the root was clamped to the cell), or
// the quadratic ENO derivative where that formula was used
__device__ void quintic_distance_jac(const double v[6], double h, double jd[6])
{
#pragma unroll
    for (int s = 0; s < 6; ++s) jd[s] = 0.0;
    if (v[1] * v[2] < 0 || v[3] * v[4] < 0) {
        using D = Dual<double, 4>;
        const D r = eno2_distance_dual<D>(D::var(v[1], 0), D::var(v[2], 1), D::var(v[3], 2), D::var(v[4], 3), h);
        for (int s = 0; s < 4; ++s) jd[s + 1] = r.d[s];
        return;
    }
    const double dist = quintic_distance(v, h);
    if (!(dist > 0.0 && dist < h)) return;
    const double t = dist + 2 * h;
    double L[6], dP = 0.0;
    for (int s = 0; s < 6; ++s) {
        double num = 1.0, den = 1.0, dnum = 0.0;
        for (int m = 0; m < 6; ++m) {
            if (m == s) continue;
            // derivative of the running product by the product rule
            dnum = dnum * (t - m * h) + num;
            num *= t - m * h;
            den *= (s - m) * h;
        }
        L[s] = num / den;
        dP += v[s] * (dnum / den);
    }
    if (dP == 0.0) return;
    for (int s = 0; s < 6; ++s) jd[s] = -L[s] / dP;
}

// W[(ax*7 + o)][c] = -(mu_fore(c) - mu_back(c + stride)) * d dist / d v[o - 1] for every
// crossed edge (c, c + stride); W is zero elsewhere (cleared by the launcher)
template <typename T>
__global__ void __launch_bounds__(128) k_adj_dist_edges(const T *__restrict__ f, EdgeLists e, Ptr6<const T> mu,
                                                          T *__restrict__ W, Grid g)
{
    for (int ax = 0; ax < 3; ++ax) {
        const unsigned n = *(e.count + ax);
        const double h = axis_h(g, ax);
        for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
            const long long c = e.idx[ax][t];
            int i, j, k;
            adj_node_of(g, c, i, j, k);
            const AxisLine L = axis_line(g, i, j, k, ax);
            const double m = (double)__ldg(mu.p[2 * ax] + c) - (double)__ldg(mu.p[2 * ax + 1] + c + L.stride);
            double v[6], jd[6];
#pragma unroll
            for (int s = -2; s <= 3; ++s) v[s + 2] = (double)__ldg(f + L.base + (long long)clampi(L.c + s, L.n) * L.stride);
            quintic_distance_jac(v, h, jd);
#pragma unroll
            for (int s = 0; s < 6; ++s) W[(long long)(ax * 7 + s + 1) * g.num + c] = (T)(-m * jd[s]);
        }
    }
}

int adj_list_blocks()
{
    static int n = 0;
    if (n == 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        n = (sms > 0 ? sms : 132) * 4;
    }
    return n;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------
template <typename T>
cudaError_t launch_adj_advect_jac(const T *ps, Ptr3<const T> v, const double *dt, const T *lam, double coef, T *W,
                                  Ptr3<T> gv, const Grid &g, cudaStream_t s)
{
    k_adj_advect_jac<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(ps, v, dt, lam, (T)coef, W, gv, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_reinit_jac(const T *ps, const uint8_t *flags, Ptr6<const T> d, const T *lam, double coef, T *W,
                                  Ptr6<T> mu, const Grid &g, cudaStream_t s)
{
    k_adj_reinit_jac<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(ps, flags, d, lam, (T)coef, W, mu, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_gather(const T *W, const T *lam, double alpha, const T *acc, T *out, const Grid &g,
                              cudaStream_t s)
{
    k_adj_gather<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(W, lam, (T)alpha, acc, out, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_axpy(T *acc, const T *lam, double a, bool init, const Grid &g, cudaStream_t s)
{
    k_adj_axpy<T><<<adj_list_blocks(), 256, 0, s>>>(acc, lam, (T)a, init, g.num);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_dist_edges(const T *f, EdgeLists e, Ptr6<const T> mu, T *W, const Grid &g, cudaStream_t s)
{
    cudaError_t err = cudaMemsetAsync(W, 0, sizeof(T) * (size_t)SLOTS * (size_t)g.num, s);
    if (err != cudaSuccess) return err;
    k_adj_dist_edges<T><<<adj_list_blocks(), 128, 0, s>>>(f, e, mu, W, g);
    return cudaGetLastError();
}

#define VSL_INSTANTIATE_ADJ(T)                                                                                     \
    template cudaError_t launch_adj_advect_jac<T>(const T *, Ptr3<const T>, const double *, const T *, double, T *, \
                                                  Ptr3<T>, const Grid &, cudaStream_t);                             \
    template cudaError_t launch_adj_reinit_jac<T>(const T *, const uint8_t *, Ptr6<const T>, const T *, double, T *, \
                                                  Ptr6<T>, const Grid &, cudaStream_t);                             \
    template cudaError_t launch_adj_gather<T>(const T *, const T *, double, const T *, T *, const Grid &,            \
                                              cudaStream_t);                                                        \
    template cudaError_t launch_adj_axpy<T>(T *, const T *, double, bool, const Grid &, cudaStream_t);              \
    template cudaError_t launch_adj_dist_edges<T>(const T *, EdgeLists, Ptr6<const T>, T *, const Grid &,          \
                                                  cudaStream_t);

VSL_INSTANTIATE_ADJ(float)
VSL_INSTANTIATE_ADJ(double)

}  // namespace vsl
