// vsl_adjoint.cu -- reverse-mode (adjoint) kernels of the WENO5 TVD-RK3 advection and
// reinitialization stages, and of the sub-cell distances the reinitialization reads.
//
// A fused stage writes  out = a * phi_n + b * (phi_s - step(phi_s)).  Its adjoint, given
// lam = dL/d out, is
//     dL/d phi_s = b * lam - J^T (b * lam),   dL/d phi_n += a * lam,
// with J the Jacobian of `step`.  Row c of J touches the 7 values of each axis line
// through c (clamped at the grid edge), so J^T is applied in two deterministic passes:
//   1. per node c, the local partials d step_c / d p_ax[o] (o = 0..6 along axis ax) are
//      evaluated -- by the closed-form gradient of the uniform WENO5 (weno5_grad), and by
//      running the forward per-node code on dual numbers where the interface is inserted
//      -- scaled by b * lam_c and stored in 21 slots W[ax*7 + o][c] (slot-major,
//      coalesced);
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

// Jiang-Shu WENO5 of five differences (the weno5_plain formula) and its gradient g[5]:
// with alpha_k = d_k / (s_k + eps)^2 and w_k = alpha_k / sum alpha,
//   dD/dv = sum_k w_k dq_k/dv + sum_k c_k ds_k/dv,   c_k = -2 w_k (q_k - D) / (s_k + eps),
// where the candidates q_k are linear and the smoothness indicators s_k quadratic in v.
template <typename T>
__device__ __forceinline__ T weno5_grad(T v1, T v2, T v3, T v4, T v5, T g[5])
{
    const T q1 = T(1. / 3.) * v1 - T(7. / 6.) * v2 + T(11. / 6.) * v3;
    const T q2 = T(-1. / 6.) * v2 + T(5. / 6.) * v3 + T(1. / 3.) * v4;
    const T q3 = T(1. / 3.) * v3 + T(5. / 6.) * v4 - T(1. / 6.) * v5;
    const T a1 = v1 - 2 * v2 + v3, b1 = v1 - 4 * v2 + 3 * v3;
    const T a2 = v2 - 2 * v3 + v4, b2 = v2 - v4;
    const T a3 = v3 - 2 * v4 + v5, b3 = 3 * v3 - 4 * v4 + v5;
    const T eps = T(1e-6);
    const T e1 = T(13. / 12.) * a1 * a1 + T(1. / 4.) * b1 * b1 + eps;
    const T e2 = T(13. / 12.) * a2 * a2 + T(1. / 4.) * b2 * b2 + eps;
    const T e3 = T(13. / 12.) * a3 * a3 + T(1. / 4.) * b3 * b3 + eps;
    const T al1 = T(0.1) / (e1 * e1), al2 = T(0.6) / (e2 * e2), al3 = T(0.3) / (e3 * e3);
    const T inv = T(1) / (al1 + al2 + al3);
    const T w1 = al1 * inv, w2 = al2 * inv, w3 = al3 * inv;
    const T D = w1 * q1 + w2 * q2 + w3 * q3;
    const T c1 = T(-2) * w1 * (q1 - D) / e1;
    const T c2 = T(-2) * w2 * (q2 - D) / e2;
    const T c3 = T(-2) * w3 * (q3 - D) / e3;
    // ds_k/dv: s1 = 13/12 a1^2 + 1/4 b1^2 with a1 = (1,-2,1,0,0).v, b1 = (1,-4,3,0,0).v, etc.
    const T A1 = T(13. / 6.) * a1 * c1, B1 = T(0.5) * b1 * c1;
    const T A2 = T(13. / 6.) * a2 * c2, B2 = T(0.5) * b2 * c2;
    const T A3 = T(13. / 6.) * a3 * c3, B3 = T(0.5) * b3 * c3;
    g[0] = T(1. / 3.) * w1 + A1 + B1;
    g[1] = T(-7. / 6.) * w1 - T(1. / 6.) * w2 - 2 * A1 - 4 * B1 + A2 + B2;
    g[2] = T(11. / 6.) * w1 + T(5. / 6.) * w2 + T(1. / 3.) * w3 + A1 + 3 * B1 - 2 * A2 + A3 + 3 * B3;
    g[3] = T(1. / 3.) * w2 + T(5. / 6.) * w3 + A2 - B2 - 2 * A3 - 4 * B3;
    g[4] = T(-1. / 6.) * w3 + A3 + B3;
    return D;
}

// Uniform WENO5 pair of one axis line (weno5_pair_plain) with its partials with respect
// to the seven line values: jf[o] = d D+ / d p[o], jb[o] = d D- / d p[o].
template <typename T>
__device__ __forceinline__ void weno5_pair_grad(const T p[7], T h, T &df, T &db, T jf[7], T jb[7])
{
    T v[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) v[m] = (p[m + 1] - p[m]) / h;
    T gb[5], gf[5];
    db = weno5_grad(v[0], v[1], v[2], v[3], v[4], gb);
    df = weno5_grad(v[5], v[4], v[3], v[2], v[1], gf);
    // G*[m] = d D / d v[m], m = 0..5
    const T Gb[6] = {gb[0], gb[1], gb[2], gb[3], gb[4], T(0)};
    const T Gf[6] = {T(0), gf[4], gf[3], gf[2], gf[1], gf[0]};
    const T ih = T(1) / h;
#pragma unroll
    for (int o = 0; o < 7; ++o) {
        const T lb = o >= 1 ? Gb[o - 1] : T(0), rb = o <= 5 ? Gb[o] : T(0);
        const T lf = o >= 1 ? Gf[o - 1] : T(0), rf = o <= 5 ? Gf[o] : T(0);
        jb[o] = (lb - rb) * ih;
        jf[o] = (lf - rf) * ih;
    }
}

// Interface-aware pair (nonuniform WENO5 with the interface inserted at r1 / l1, value 0)
// and its partials with respect to the seven line values (0..6) and r1, l1 (7, 8), by
// dual numbers; out of line, since only the few band nodes take it.
template <typename T>
__device__ __noinline__ void iface_pair_jac(const T p[7], T h, T r1, T l1, T &df, T &db, T jf[9], T jb[9])
{
    using D = Dual<T, 9>;
    D P[7];
#pragma unroll
    for (int o = 0; o < 7; ++o) P[o] = D::var(p[o], o);
    D f, b;
    interface_pair<D>(P, D::var(r1, 7), D::var(l1, 8), D((double)h), D(0.0), D(0.0), false, f, b);
    df = f.v;
    db = b.v;
#pragma unroll
    for (int o = 0; o < 9; ++o) {
        jf[o] = f.d[o];
        jb[o] = b.d[o];
    }
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
        T p[7], jf[7], jb[7], df, db;
        load_line7(ps, axis_line(g, i, j, k, ax), p);
        weno5_pair_grad<T>(p, (T)axis_h(g, ax), df, db, jf, jb);
        const T va = __ldg(v.p[ax] + c);
        const T vm = vmin(T(0), va), vp = vmax(T(0), va);
#pragma unroll
        for (int o = 0; o < 7; ++o) W[(long long)(ax * 7 + o) * g.num + c] = lc * (vm * jf[o] + vp * jb[o]);
        // d step / d v: D- where v > 0, D+ otherwise (the branches of max/min above)
        gv.p[ax][c] -= lc * (va > T(0) ? db : df);
    }
}

// ---------------------------------------------------------------------------------------
// reinitialization stage: step = (|grad|_Godunov - 1) * 0.3 min(dist) * (mask ? -1 : 1)
// ---------------------------------------------------------------------------------------
// One node of the reinitialization-stage Jacobian.  GENERIC = false handles only nodes
// whose three axis lines are all uniform (no sign change next to the node); GENERIC =
// true also differentiates the interface-aware pairs (dual numbers) and is run over the
// compact list of the remaining nodes, so the register cost of the dual code does not
// limit the occupancy of the dense pass.
template <typename T, bool GENERIC>
__device__ __forceinline__ void reinit_jac_node(const T *__restrict__ ps, const uint8_t fl, Ptr6<const T> d,
                                                const T lc, T *__restrict__ W, Ptr6<T> mu, const Grid &g, int i,
                                                int j, int k, long long c)
{
    const T h[3] = {(T)g.dx, (T)g.dy, (T)g.dz};
    // the six distances (stored where flagged, the spacing elsewhere); the pseudo-time
    // step is 0.3 * their minimum, taken in the order of the forward kernel's vmin tree
    T dist[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) dist[q] = (fl & (1u << q)) ? __ldg(d.p[q] + c) : h[q / 2];
    const int i01 = dist[0] < dist[1] ? 0 : 1, i23 = dist[2] < dist[3] ? 2 : 3, i45 = dist[4] < dist[5] ? 4 : 5;
    const int i25 = dist[i23] < dist[i45] ? i23 : i45;
    const int qmin = dist[i01] < dist[i25] ? i01 : i25;
    const T dtv = T(0.3) * dist[qmin];
    const bool neg = fl & CLS_MASK;
    const T sgn = neg ? T(-1) : T(1);

    // pass 1: the derivative pairs and the partials of the Godunov norm
    //   G = sqrt(sum_ax max(A_ax, B_ax)) with the branch of each max as the forward took it
    bool iface[3];
    T gq[6], S = T(0);
    const T z = T(0);
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
        T p[7], df, db;
        load_line7(ps, axis_line(g, i, j, k, ax), p);
        iface[ax] = GENERIC && (p[2] * p[3] < T(0) || p[3] * p[4] < T(0));
        if (GENERIC && iface[ax])
            interface_pair<T>(p, dist[2 * ax], dist[2 * ax + 1], h[ax], T(0), T(0), false, df, db);
        else
            weno5_pair_plain<T>(p, h[ax], df, db);
        const T A = neg ? sqr(vmin(z, db)) : sqr(vmax(z, db));
        const T B = neg ? sqr(vmax(z, df)) : sqr(vmin(z, df));
        if (A < B) {  // vmax(A, B) took B (the forward derivative)
            S += B;
            gq[2 * ax] = T(2) * (neg ? vmax(z, df) : vmin(z, df));
            gq[2 * ax + 1] = T(0);
        } else {
            S += A;
            gq[2 * ax] = T(0);
            gq[2 * ax + 1] = T(2) * (neg ? vmin(z, db) : vmax(z, db));
        }
    }
    const T G = sqrt(S);
    const T dG = G > T(0) ? T(0.5) / G : T(0);  // zero derivative of sqrt at 0
    const T s_dt = dtv * sgn;

    // pass 2: per axis, partials of the pair, scaled into the slots and distance adjoints
    T md[6];
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
        T p[7], jf[9], jb[9], df, db;
        load_line7(ps, axis_line(g, i, j, k, ax), p);
        if constexpr (GENERIC) {
            if (iface[ax]) {
                iface_pair_jac<T>(p, h[ax], dist[2 * ax], dist[2 * ax + 1], df, db, jf, jb);
            } else {
                weno5_pair_grad<T>(p, h[ax], df, db, jf, jb);
                jf[7] = jf[8] = jb[7] = jb[8] = T(0);
            }
        } else {
            weno5_pair_grad<T>(p, h[ax], df, db, jf, jb);
            jf[7] = jf[8] = jb[7] = jb[8] = T(0);
        }
        const T gf = gq[2 * ax] * dG * s_dt, gb = gq[2 * ax + 1] * dG * s_dt;
#pragma unroll
        for (int o = 0; o < 7; ++o) W[(long long)(ax * 7 + o) * g.num + c] = lc * (gf * jf[o] + gb * jb[o]);
        md[2 * ax] = gf * jf[7] + gb * jb[7];
        md[2 * ax + 1] = gf * jf[8] + gb * jb[8];
    }
    // d step / d dist_q: through the interface insertion, and through dt for the minimum
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        if (!(fl & (1u << q))) continue;
        const T ds = md[q] + (q == qmin ? (G - T(1)) * sgn * T(0.3) : T(0));
        mu.p[q][c] -= lc * ds;
    }
}

// warp-aggregated append of `value` where `pred` holds (all 32 lanes of the warp call it)
__device__ __forceinline__ void adj_append(bool pred, unsigned value, unsigned *list, unsigned *count)
{
    const unsigned m = __ballot_sync(0xffffffffu, pred);
    if (!m) return;
    const unsigned lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31u;
    const int leader = __ffs(m) - 1;
    unsigned base = 0;
    if ((int)lane == leader) base = atomicAdd(count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pred) list[base + __popc(m & ((1u << lane) - 1u))] = value;
}

// dense pass: fixed nodes get zero slots; nodes with a sign change next to them on any
// axis are listed for k_adj_reinit_jac_band; the rest are done here
template <typename T>
__global__ void __launch_bounds__(BX *BY) k_adj_reinit_jac(const T *__restrict__ ps, const uint8_t *__restrict__ flags,
                                                             Ptr6<const T> d, const T *__restrict__ lam, T coef,
                                                             T *__restrict__ W, Ptr6<T> mu, NodeList band, Grid g)
{
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z;
    const bool in = i < g.rows && j < g.cols;
    const long long c = in ? node_index(g, i, j, k) : 0;
    const uint8_t fl = in ? __ldg(flags + c) : uint8_t(0);
    bool near = false;
    if (in && !(fl & CLS_FIXED)) {
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const AxisLine L = axis_line(g, i, j, k, ax);
            const T pm = __ldg(ps + L.base + (long long)clampi(L.c - 1, L.n) * L.stride);
            const T p0 = __ldg(ps + c);
            const T pp = __ldg(ps + L.base + (long long)clampi(L.c + 1, L.n) * L.stride);
            near |= pm * p0 < T(0) || p0 * pp < T(0);
        }
    }
    adj_append(near, (unsigned)c, band.idx, band.count);
    if (!in || near) return;
    if (fl & CLS_FIXED) {
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) W[(long long)s * g.num + c] = T(0);
        return;
    }
    reinit_jac_node<T, false>(ps, fl, d, coef * __ldg(lam + c), W, mu, g, i, j, k, c);
}

template <typename T>
__global__ void __launch_bounds__(128) k_adj_reinit_jac_band(const T *__restrict__ ps,
                                                               const uint8_t *__restrict__ flags, Ptr6<const T> d,
                                                               const T *__restrict__ lam, T coef, T *__restrict__ W,
                                                               Ptr6<T> mu, NodeList band, Grid g)
{
    const unsigned n = *band.count;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const long long c = band.idx[t];
        int i, j, k;
        adj_node_of(g, c, i, j, k);
        reinit_jac_node<T, true>(ps, __ldg(flags + c), d, coef * __ldg(lam + c), W, mu, g, i, j, k, c);
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
                                  Ptr6<T> mu, NodeList band, const Grid &g, cudaStream_t s)
{
    cudaError_t err = cudaMemsetAsync(band.count, 0, sizeof(unsigned), s);
    if (err != cudaSuccess) return err;
    k_adj_reinit_jac<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(ps, flags, d, lam, (T)coef, W, mu, band, g);
    k_adj_reinit_jac_band<T><<<adj_list_blocks(), 128, 0, s>>>(ps, flags, d, lam, (T)coef, W, mu, band, g);
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
                                                  Ptr6<T>, NodeList, const Grid &, cudaStream_t);                   \
    template cudaError_t launch_adj_gather<T>(const T *, const T *, double, const T *, T *, const Grid &,            \
                                              cudaStream_t);                                                        \
    template cudaError_t launch_adj_axpy<T>(T *, const T *, double, bool, const Grid &, cudaStream_t);              \
    template cudaError_t launch_adj_dist_edges<T>(const T *, EdgeLists, Ptr6<const T>, T *, const Grid &,          \
                                                  cudaStream_t);

VSL_INSTANTIATE_ADJ(float)
VSL_INSTANTIATE_ADJ(double)

}  // namespace vsl
