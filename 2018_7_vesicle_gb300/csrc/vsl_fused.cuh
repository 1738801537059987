// vsl_fused.cuh -- fused TVD-RK3 stage kernels of the method-level operations, included
// by vsl_fused_f64.cu (plain form, compiled without multiply-add contraction so that the
// FP64 arithmetic rounds like the reference's) and vsl_fused_f32.cu (mixed form).
//
// One launch evaluates one Runge-Kutta stage of a whole pseudo-step AND its Shu-Osher
// combination, writing the next stage field directly:
//   stage 0: out = phi_s - step(phi_s)
//   stage 1: out = 3/4 phi_n + 1/4 (phi_s - step(phi_s))
//   stage 2: out = 1/3 phi_n + 2/3 (phi_s - step(phi_s))
// which are the elementwise updates of WENO5RK3Reinitialization.m:15-39 (and of the
// extension loops) folded into the stencil pass.
//
// Per node, a classification byte written once per call replaces the six distance reads:
//   bits 0..5  distance xpr,xpl,ypf,ypb,zpu,zpd differs from the grid spacing (crossing)
//   bit  6     mask (phi < 0 when the call started)
//   bit  7     fixed node (a distance below 1e-6*dx: the reference's step-0 nodes)
// Distances and crossing values are read only where a bit says they differ from the
// defaults, so the dense per-stage traffic is phi_s (stencil), phi_n, flags and out.
#pragma once

#include <math_constants.h>
#include <type_traits>

#include "vsl_internal.h"

namespace vsl {
namespace {

constexpr uint8_t FIXED_BIT = 0x80;
constexpr uint8_t MASK_BIT = 0x40;

__device__ __forceinline__ bool fused_node(const Grid &g, int &i, int &j, int &k)
{
    i = blockIdx.x * BX + threadIdx.x;
    j = blockIdx.y * BY + threadIdx.y;
    k = blockIdx.z;
    return i < g.rows && j < g.cols;
}

template <typename T> __device__ __forceinline__ T rk3_combine(int stage, T phi_n, T t)
{
    if (stage == 0) return t;
    if (stage == 1) return T(3. / 4.) * phi_n + T(1. / 4.) * t;
    return T(1. / 3.) * phi_n + T(2. / 3.) * t;
}

// distance of direction q (0..5) at node c: the stored value where the flag says it
// differs from the spacing, the spacing otherwise
template <typename T>
__device__ __forceinline__ T flagged_distance(uint8_t fl, int q, const Ptr6<const T> &d, long long c, T h)
{
    return (fl & (1u << q)) ? __ldg(d.p[q] + c) : h;
}

// 0.3 * min over the six distances, as deltat = 0.3*min_dist of setDistance.m:17-21
template <typename T>
__device__ __forceinline__ T pseudo_dt(uint8_t fl, const Ptr6<const T> &d, long long c, T hx, T hy, T hz)
{
    T v[6];
    const T h[3] = {hx, hy, hz};
#pragma unroll
    for (int q = 0; q < 6; ++q) v[q] = flagged_distance(fl, q, d, c, h[q / 2]);
    T m = vmin(vmin(v[0], v[1]), vmin(vmin(v[2], v[3]), vmin(v[4], v[5])));
    return T(0.3) * m;
}

template <typename T, bool FAST>
__device__ __forceinline__ void uniform_pair(const T p[7], T h, T &df, T &db)
{
    if (FAST) {
        const T inv_h = T(1) / h;
        const T eps2 = T(1e-6) * h * h;
        weno5_pair_fast(p, inv_h, eps2, df, db);
    } else {
        weno5_pair_plain(p, h, df, db);
    }
}

// warp-aggregated append of `value` to a device list where `pred` holds (all 32 lanes of
// the warp must call it)
__device__ __forceinline__ void warp_append(bool pred, unsigned value, unsigned *list, unsigned *count)
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

__device__ __forceinline__ void node_of(const Grid &g, long long c, int &i, int &j, int &k)
{
    k = (int)(c / g.plane);
    const long long r = c - (long long)k * g.plane;
    j = (int)(r / g.rows);
    i = (int)(r - (long long)j * g.rows);
}

// ---------------------------------------------------------------------------------------
// setDistance (setDistance.m:5-15 with boundary_location.cu:84-132 / boundary_correction):
// pass 1 writes the spacing everywhere and lists every edge (c, c+1) the zero set crosses;
// pass 2 solves one root per listed edge and writes both of its endpoint distances
// (h minus it on the far side), the values of the reference's scatter form.
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(BX *BY) k_dist_scan(const T *__restrict__ f, Ptr6<T> d, EdgeLists e, Grid g)
{
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z;
    const bool in = i < g.rows && j < g.cols;
    const long long c = in ? node_index(g, i, j, k) : 0;
    const T f0 = in ? __ldg(f + c) : T(0);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        bool cross = false;
        if (in) {
            AxisLine L = axis_line(g, i, j, k, ax);
            const T h = (T)axis_h(g, ax);
            d.p[2 * ax][c] = h;
            d.p[2 * ax + 1][c] = h;
            const T fn = __ldg(f + L.base + (long long)clampi(L.c + 1, L.n) * L.stride);
            // the reference's test f0 * fn < 0 in FP64; for FP32 inputs the FP64 product of
            // two nonzero values never underflows, so it is exactly the sign test below
            if constexpr (std::is_same<T, float>::value)
                cross = (f0 > T(0) && fn < T(0)) || (f0 < T(0) && fn > T(0));
            else
                cross = f0 * fn < 0;
        }
        warp_append(cross, (unsigned)c, e.idx[ax], e.count + ax);
    }
}

template <typename T, bool QUINTIC>
__global__ void __launch_bounds__(128) k_dist_roots(const T *__restrict__ f, Ptr6<T> d, EdgeLists e, Grid g)
{
    // the three axes' lists as one, so that a thread solves one root rather than one per axis
    const unsigned n0 = e.count[0], n01 = n0 + e.count[1], n = n01 + e.count[2];
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int ax = t < n0 ? 0 : (t < n01 ? 1 : 2);
        const long long c = e.idx[ax][t - (ax == 0 ? 0u : (ax == 1 ? n0 : n01))];
        const double h = axis_h(g, ax);
        int i, j, k;
        node_of(g, c, i, j, k);
        const AxisLine L = axis_line(g, i, j, k, ax);
        const double dist = fore_distance<QUINTIC>(f, L, h);
        d.p[2 * ax][c] = (T)dist;
        d.p[2 * ax + 1][c + L.stride] = (T)(h - dist);
    }
}

template <typename T>
__global__ void __launch_bounds__(BX *BY) k_classify(const T *__restrict__ phi0, Ptr6<const T> d, uint8_t *flags,
                                                      NodeList list, Grid g)
{
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z;
    const bool in = i < g.rows && j < g.cols;
    const long long c = in ? node_index(g, i, j, k) : 0;
    uint8_t fl = 0;
    if (in) {
        const T h[3] = {(T)g.dx, (T)g.dy, (T)g.dz};
        const T tiny = (T)(1e-6 * g.dx);
        bool fixed = false;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const T v = __ldg(d.p[q] + c);
            if (v != h[q / 2]) fl |= (uint8_t)(1u << q);
            fixed |= v < tiny;
        }
        if (__ldg(phi0 + c) < T(0)) fl |= MASK_BIT;
        if (fixed) fl |= FIXED_BIT;
        flags[c] = fl;
    }
    if (list.idx) warp_append((fl & 0x3F) != 0, (unsigned)c, list.idx, list.count);
}

// The FP32 classification with four consecutive nodes per thread: the classification is
// elementwise in the linear index, so the field and the six distances are read as 16-byte
// vectors and the four flag bytes written as one word (node count a multiple of 4, every
// array 16-byte aligned; the launcher checks).  The flags are k_classify's.
__global__ void __launch_bounds__(256) k_classify4(const float *__restrict__ phi0, Ptr6<const float> d,
                                                   uint8_t *flags, NodeList list, long long n4, float hx, float hy,
                                                   float hz, float tiny)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = t < n4;
    const float h[3] = {hx, hy, hz};
    uint8_t fl[4] = {0, 0, 0, 0};
    if (in) {
        bool fixed[4] = {false, false, false, false};
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float4 v = __ldg(reinterpret_cast<const float4 *>(d.p[q]) + t);
            const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                if (e[r] != h[q / 2]) fl[r] |= (uint8_t)(1u << q);
                fixed[r] |= e[r] < tiny;
            }
        }
        const float4 f = __ldg(reinterpret_cast<const float4 *>(phi0) + t);
        const float fv[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (fv[r] < 0.f) fl[r] |= MASK_BIT;
            if (fixed[r]) fl[r] |= FIXED_BIT;
        }
        reinterpret_cast<uchar4 *>(flags)[t] = make_uchar4(fl[0], fl[1], fl[2], fl[3]);
    }
    if (list.idx) {
        // append the flagged nodes in node order (as k_classify's warps do): a warp-wide
        // exclusive scan of the per-lane counts, one atomic per warp
        const unsigned lane = threadIdx.x & 31u;
        unsigned mine = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r) mine += (fl[r] & 0x3F) ? 1u : 0u;
        unsigned incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += y;
        }
        const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
        if (total) {
            unsigned base = 0;
            if (lane == 31) base = atomicAdd(list.count, total);
            base = __shfl_sync(0xffffffffu, base, 31) + incl - mine;
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (fl[r] & 0x3F) list.idx[base++] = (unsigned)(4 * t + r);
        }
    }
}

// The short gaps beyond the crossings of node c on line L (FP32 distances): h - r1 and
// h - l1 as the neighbours beyond the crossings store them (their own distance, h - dist
// rounded once from the FP64 root), where they agree with h - r1 / h - l1 to 1e-6 h (so
// distances from any source stay safe); h - r1 / h - l1 otherwise and at the line's ends.
__device__ __forceinline__ void crossing_gaps(const AxisLine &L, int ax, const Ptr6<const float> &d, long long c,
                                              float r1, float l1, float h, float &rc, float &lc)
{
    rc = h - r1;
    lc = h - l1;
    if (r1 < h && L.c + 1 < L.n) {
        const float nb = __ldg(d.p[2 * ax + 1] + c + L.stride);
        if (fabsf(r1 + nb - h) <= 1e-6f * h) rc = nb;
    }
    if (l1 < h && L.c > 0) {
        const float nb = __ldg(d.p[2 * ax] + c - L.stride);
        if (fabsf(l1 + nb - h) <= 1e-6f * h) lc = nb;
    }
}

// The interface-aware pair at node c of axis line L (r1 / l1: the node's distances, hf /
// hb: the values at the crossings).  The plain FP64 form takes the reference's position
// form.  The mixed FP32 form takes the gap form with the short gaps of crossing_gaps.
template <typename T, bool ENO3>
__device__ __forceinline__ void node_interface_pair(const T p[7], const AxisLine &L, int ax, const Ptr6<const T> &d,
                                                    long long c, T r1, T l1, T h, T hf, T hb, T &df, T &db)
{
    if constexpr (std::is_same<T, float>::value) {
        T rc, lc;
        crossing_gaps(L, ax, d, c, r1, l1, h, rc, lc);
        interface_pair_gaps(p, r1, rc, l1, lc, h, hf, hb, ENO3, df, db);
    } else {
        interface_pair(p, r1, l1, h, hf, hb, ENO3, df, db);
    }
}

// ---------------------------------------------------------------------------------------
// reinitialization stage (re_step.cu:283-393 / weno_rk3_reinitialization.cu:295-406)
// ---------------------------------------------------------------------------------------
// one node of a reinitialization stage, all reads from global memory (clamped)
template <typename T, bool ENO3, bool FAST>
__device__ __forceinline__ void reinit_node(const T *__restrict__ phi_s, const T *__restrict__ phi_n,
                                            T *__restrict__ out, const uint8_t *__restrict__ flags,
                                            const Ptr6<const T> &d, const Grid &g, int stage, int i, int j, int k)
{
    const long long c = node_index(g, i, j, k);
    const uint8_t fl = __ldg(flags + c);
    const T ps = __ldg(phi_s + c);
    const T hx = (T)g.dx, hy = (T)g.dy, hz = (T)g.dz;
    T step = T(0);
    if (!(fl & FIXED_BIT)) {
        T df[3], db[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            T p[7];
            const AxisLine L = axis_line(g, i, j, k, ax);
            load_line7(phi_s, L, p);
            const T h = ax == 0 ? hx : (ax == 1 ? hy : hz);
            if (p[2] * p[3] < T(0) || p[3] * p[4] < T(0)) {
                const T r1 = flagged_distance(fl, 2 * ax, d, c, h);
                const T l1 = flagged_distance(fl, 2 * ax + 1, d, c, h);
                node_interface_pair<T, ENO3>(p, L, ax, d, c, r1, l1, h, T(0), T(0), df[ax], db[ax]);
            } else {
                uniform_pair<T, FAST>(p, h, df[ax], db[ax]);
            }
        }
        const bool neg = fl & MASK_BIT;
        const T gn = godunov_norm(neg, df[0], db[0], df[1], db[1], df[2], db[2]);
        step = (gn - T(1)) * pseudo_dt(fl, d, c, hx, hy, hz) * (neg ? T(-1) : T(1));
    }
    const T pn = stage == 0 ? T(0) : __ldg(phi_n + c);
    out[c] = rk3_combine(stage, pn, ps - step);
}

template <typename T, bool ENO3, bool FAST>
__global__ void __launch_bounds__(BX *BY) k_reinit_stage(const T *__restrict__ phi_s, const T *__restrict__ phi_n,
                                                           T *__restrict__ out, const uint8_t *__restrict__ flags,
                                                           Ptr6<const T> d, Grid g, int stage)
{
    int i, j, k;
    if (!fused_node(g, i, j, k)) return;
    reinit_node<T, ENO3, FAST>(phi_s, phi_n, out, flags, d, g, stage, i, j, k);
}

// ---------------------------------------------------------------------------------------
// reinitialization residual
// ---------------------------------------------------------------------------------------
// | |grad phi|_G - 1 | at node c in FP64 (the Godunov norm of re_step.cu:382-392 with the
// stage's stencil choice: the interface-aware pair where the line changes sign).  The plain
// form takes reinit_node's FP64 arithmetic; the mixed form promotes its FP32 values and
// takes the gap form of its distances.
template <typename T>
__device__ __forceinline__ double residual_node(const T *__restrict__ phi, uint8_t fl, const Ptr6<const T> &d,
                                                const Grid &g, int i, int j, int k, long long c)
{
    double df[3], db[3];
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
        const AxisLine L = axis_line(g, i, j, k, ax);
        T pt[7];
        load_line7(phi, L, pt);
        double p[7];
#pragma unroll
        for (int m = 0; m < 7; ++m) p[m] = (double)pt[m];
        const double h = axis_h(g, ax);
        if (p[2] * p[3] < 0.0 || p[3] * p[4] < 0.0) {
            if constexpr (std::is_same<T, float>::value) {
                const float hf = (float)h;
                const float r1 = flagged_distance(fl, 2 * ax, d, c, hf), l1 = flagged_distance(fl, 2 * ax + 1, d, c, hf);
                float rc, lc;
                crossing_gaps(L, ax, d, c, r1, l1, hf, rc, lc);
                interface_pair_gaps<double>(p, r1, rc, l1, lc, hf, 0.0, 0.0, false, df[ax], db[ax]);
            } else {
                const double r1 = flagged_distance(fl, 2 * ax, d, c, h), l1 = flagged_distance(fl, 2 * ax + 1, d, c, h);
                interface_pair<double>(p, r1, l1, h, 0.0, 0.0, false, df[ax], db[ax]);
            }
        } else {
            weno5_pair_plain<double>(p, h, df[ax], db[ax]);
        }
    }
    const double gn = godunov_norm((fl & MASK_BIT) != 0, df[0], db[0], df[1], db[1], df[2], db[2]);
    return fabs(gn - 1.0);
}

template <typename T>
__global__ void __launch_bounds__(BX *BY) k_reinit_residual(const T *__restrict__ phi, const uint8_t *__restrict__ flags,
                                                              Ptr6<const T> d, Grid g, double band, ResidualState st)
{
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y, k = blockIdx.z;
    double r = 0.0;
    if (i < g.rows && j < g.cols) {
        const long long c = node_index(g, i, j, k);
        const uint8_t fl = __ldg(flags + c);
        if (fabs((double)__ldg(phi + c)) < band && !(fl & FIXED_BIT)) r = residual_node<T>(phi, fl, d, g, i, j, k, c);
        if (r != r) r = CUDART_INF;  // a NaN never counts as converged
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_down_sync(0xffffffffu, r, o));
    __shared__ double sm[BX * BY / 32];
    const int t = threadIdx.y * BX + threadIdx.x;
    if ((t & 31) == 0) sm[t >> 5] = r;
    __syncthreads();
    if (t != 0) return;
    for (int w = 1; w < BX * BY / 32; ++w) r = fmax(r, sm[w]);
    // non-negative doubles order as their bit patterns
    atomicMax(st.max_bits, (unsigned long long)__double_as_longlong(r));
    __threadfence();
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    if (atomicAdd(st.ticket, 1u) != nb - 1) return;
    // the last block: every other block's maximum is in (each fenced before its ticket)
    const double res = __longlong_as_double((long long)atomicExch(st.max_bits, 0ull));
    *st.ticket = 0u;
    const int it = st.status[0] + st.advance;
    st.status[0] = it;
    if (st.history) st.history[it] = res;
    const bool conv = res <= st.tol;
    st.status[1] = conv ? 1 : 0;
    if (st.zero_counter) *st.zero_counter = 0u;
    if (st.has_handle) cudaGraphSetConditional(st.handle, (!conv && it < st.cap) ? 1u : 0u);
}

__global__ void k_condition_reset(cudaGraphConditionalHandle handle) { cudaGraphSetConditional(handle, 0u); }

// ---------------------------------------------------------------------------------------
// extension set-up: v = sign(F) * grad / max(|grad|, floor) with the upwind normal of
// upwind_normal.cu:4-104 (WENORK3: wenork3_extend.cu:192-292) and the normalisation of
// WENO5RK3Extend.m:23-31
// ---------------------------------------------------------------------------------------
// The classification byte says which distances differ from the spacing (only those are
// read); away from the interface the mixed form takes the packed fast WENO5 pair.
// one node of the extension velocity (the generic form: interface-aware one-sided
// derivatives on the axes with a crossing)
template <typename T, bool ENO3>
__device__ __forceinline__ void extension_velocity_node(const T *__restrict__ phi, const uint8_t *__restrict__ flags,
                                                        const Ptr6<const T> &d, Ptr3<T> &v, const Grid &g, T floor,
                                                        int i, int j, int k)
{
    const long long c = node_index(g, i, j, k);
    const uint8_t fl = __ldg(flags + c);
    T n[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        T p[7], df, db;
        const AxisLine L = axis_line(g, i, j, k, ax);
        load_line7(phi, L, p);
        const T h = (T)axis_h(g, ax);
        const T r1 = flagged_distance(fl, 2 * ax, d, c, h), l1 = flagged_distance(fl, 2 * ax + 1, d, c, h);
        if (r1 < h || l1 < h) {
            node_interface_pair<T, ENO3>(p, L, ax, d, c, r1, l1, h, T(0), T(0), df, db);
        } else {
            if constexpr (std::is_same<T, float>::value)
                weno5_pair_fast2(p, 1.0f / h, 1e-6f * h * h, df, db);
            else
                weno5_pair_plain(p, h, df, db);
        }
        n[ax] = (fabs(p[4]) < fabs(p[2])) ? df : db;
    }
    const T grad = vmax(sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]), floor);
    const T f0 = __ldg(phi + c);
    const T s = f0 > T(0) ? T(1) : (f0 < T(0) ? T(-1) : T(0));
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) v.p[ax][c] = s * (n[ax] / grad);
}

template <typename T, bool ENO3>
__global__ void __launch_bounds__(BX *BY) k_extension_velocity(const T *__restrict__ phi,
                                                                 const uint8_t *__restrict__ flags, Ptr6<const T> d,
                                                                 Ptr3<T> v, Grid g, T floor)
{
    int i, j, k;
    if (!fused_node(g, i, j, k)) return;
    extension_velocity_node<T, ENO3>(phi, flags, d, v, g, floor, i, j, k);
}

// The mixed form splits the extension velocity: nodes without a distance flag take the
// uniform path on 2.5D tiles (stage kind SK_VELOCITY), where only the side each axis keeps
// (n = D+ where |p4| < |p2|, else D-) is reconstructed, x and y as the two lanes of one
// packed WENO5, z with itself in both lanes; each lane is the arithmetic of the
// corresponding lane of weno5_pair_fast2, so the velocity is the same to the bit.  The
// flagged nodes (the classification's list) run the generic form in k_velocity_list.

// the flagged nodes of the extension velocity (the classification's list), generic form
template <bool ENO3>
__global__ void __launch_bounds__(128) k_velocity_list(const float *__restrict__ phi, const uint8_t *__restrict__ flags,
                                                       Ptr6<const float> d, Ptr3<float> v, NodeList list, Grid g,
                                                       float floor)
{
    const unsigned n = *list.count;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const long long c = list.idx[t];
        int i, j, k;
        node_of(g, c, i, j, k);
        extension_velocity_node<float, ENO3>(phi, flags, d, v, g, floor, i, j, k);
    }
}

// crossing values (boundary_interpolant.cu:78-141 / wenork3_extend.cu:296-365), at the
// listed nodes only (a node without a distance flag has no crossing, and its entries are
// never read): the reference's FP64 construction (the mixed form's extension takes its
// FP64 crossing values from k_crossing_mixed)
template <typename T, bool CUBIC>
__global__ void __launch_bounds__(128) k_crossing(const T *__restrict__ cfield, Ptr6<const T> d, Ptr6<T> cp,
                                                  NodeList list, Grid g)
{
    const unsigned n = *list.count;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const long long c = list.idx[t];
        int i, j, k;
        node_of(g, c, i, j, k);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const double h = axis_h(g, ax);
            const double r1 = (double)__ldg(d.p[2 * ax] + c), l1 = (double)__ldg(d.p[2 * ax + 1] + c);
            double cf = 0.0, cb = 0.0;
            if (r1 < h || l1 < h) {
                AxisLine L = axis_line(g, i, j, k, ax);
                double p[7];
#pragma unroll
                for (int s = -3; s <= 3; ++s)
                    p[s + 3] = (double)__ldg(cfield + L.base + (long long)clampi(L.c + s, L.n) * L.stride);
                if (CUBIC)
                    crossing_cubic(p, r1, l1, h, cf, cb);
                else
                    crossing_quintic(p, r1, l1, h, cf, cb);
            }
            cp.p[2 * ax][c] = (T)cf;
            cp.p[2 * ax + 1][c] = (T)cb;
        }
    }
}

// ---------------------------------------------------------------------------------------
// extension stage (extend_step.cu:10-125 / wenork3_extend.cu:372-487)
// ---------------------------------------------------------------------------------------
// one node of an extension stage, all reads from global memory (clamped)
template <typename T, bool ENO3, bool FAST>
__device__ __forceinline__ void extend_node(const T *__restrict__ c_s, const T *__restrict__ c_n, T *__restrict__ out,
                                            const uint8_t *__restrict__ flags, const Ptr6<const T> &d,
                                            const Ptr6<const T> &cp, const Ptr3<const T> &v, const Grid &g, int stage,
                                            int i, int j, int k)
{
    const long long c = node_index(g, i, j, k);
    const uint8_t fl = __ldg(flags + c);
    const T cs = __ldg(c_s + c);
    const T hx = (T)g.dx, hy = (T)g.dy, hz = (T)g.dz;
    T step = T(0);
    if (!(fl & FIXED_BIT)) {
        T df[3], db[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            T p[7];
            const AxisLine L = axis_line(g, i, j, k, ax);
            load_line7(c_s, L, p);
            const T h = ax == 0 ? hx : (ax == 1 ? hy : hz);
            const T r1 = flagged_distance(fl, 2 * ax, d, c, h);
            const T l1 = flagged_distance(fl, 2 * ax + 1, d, c, h);
            if (r1 < h || l1 < h) {
                const T hf = r1 < h ? __ldg(cp.p[2 * ax] + c) : T(0);
                const T hb = l1 < h ? __ldg(cp.p[2 * ax + 1] + c) : T(0);
                node_interface_pair<T, ENO3>(p, L, ax, d, c, r1, l1, h, hf, hb, df[ax], db[ax]);
            } else {
                uniform_pair<T, FAST>(p, h, df[ax], db[ax]);
            }
        }
        step = upwind_dot(__ldg(v.p[0] + c), __ldg(v.p[1] + c), __ldg(v.p[2] + c), df[0], db[0], df[1], db[1], df[2],
                          db[2]) *
               pseudo_dt(fl, d, c, hx, hy, hz);
    }
    const T pn = stage == 0 ? T(0) : __ldg(c_n + c);
    out[c] = rk3_combine(stage, pn, cs - step);
}

template <typename T, bool ENO3, bool FAST>
__global__ void __launch_bounds__(BX *BY) k_extend_stage(const T *__restrict__ c_s, const T *__restrict__ c_n,
                                                           T *__restrict__ out, const uint8_t *__restrict__ flags,
                                                           Ptr6<const T> d, Ptr6<const T> cp, Ptr3<const T> v, Grid g,
                                                           int stage)
{
    int i, j, k;
    if (!fused_node(g, i, j, k)) return;
    extend_node<T, ENO3, FAST>(c_s, c_n, out, flags, d, cp, v, g, stage, i, j, k);
}

// ---------------------------------------------------------------------------------------
// WENO5 advection stage: step = dt * (upwind v.grad phi) (advection_step.cu:30-56).
// With `speed` non-null the velocity is speed * (v0, v1, v2) (normal speed times normal).
// ---------------------------------------------------------------------------------------
template <typename T, bool FAST>
__global__ void __launch_bounds__(BX *BY) k_advect_stage(const T *__restrict__ phi_s, const T *__restrict__ phi_n,
                                                           T *__restrict__ out, Ptr3<const T> v,
                                                           const T *__restrict__ speed, const double *__restrict__ dt,
                                                           Grid g, int stage)
{
    int i, j, k;
    if (!fused_node(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    T df[3], db[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        T p[7];
        load_line7(phi_s, axis_line(g, i, j, k, ax), p);
        uniform_pair<T, FAST>(p, (T)axis_h(g, ax), df[ax], db[ax]);
    }
    T vx = __ldg(v.p[0] + c), vy = __ldg(v.p[1] + c), vz = __ldg(v.p[2] + c);
    if (speed) {
        const T sp = __ldg(speed + c);
        vx = sp * vx;
        vy = sp * vy;
        vz = sp * vz;
    }
    const T step = (T)__ldg(dt) * upwind_dot(vx, vy, vz, df[0], db[0], df[1], db[1], df[2], db[2]);
    const T pn = stage == 0 ? T(0) : __ldg(phi_n + c);
    out[c] = rk3_combine(stage, pn, __ldg(phi_s + c) - step);
}

// ---------------------------------------------------------------------------------------
// ENORK2 (second-order ENO with the sub-cell fix, Heun RK2): ENORK2Reinitialization.m:3-45
// and ENORK2Extend.m:9-81 over the kernels of boundary_correction.cu and enork2_extend.cu.
// The fused stage writes
//   stage 0: out = phi_s - step(phi_s)
//   stage 1: out = (phi_n + phi_s - step(phi_s)) / 2      (the reinitialization and
//            extension loops)
//   stage 2: out = (phi_n + (phi_s - step(phi_s))) / 2    (the closest-point surface
//            redistance, ENORK2ClosetPointSurfaceRedistance.m:96-100)
// the elementwise updates of the MATLAB loops in their rounding order.  There is no
// fixed-node test.
// ---------------------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T rk2_combine(int stage, T phi_n, T phi_s, T step)
{
    if (stage == 0) return phi_s - step;
    if (stage == 1) return (phi_n + phi_s - step) / T(2);
    return (phi_n + (phi_s - step)) / T(2);
}

// one quadratic-ENO root per listed crossed edge (k_dist_roots with the ENORK2 distance)
template <typename T>
__global__ void __launch_bounds__(128) k_dist_roots_eno2(const T *__restrict__ f, Ptr6<T> d, EdgeLists e, Grid g)
{
    const unsigned n0 = e.count[0], n01 = n0 + e.count[1], n = n01 + e.count[2];
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int ax = t < n0 ? 0 : (t < n01 ? 1 : 2);
        const long long c = e.idx[ax][t - (ax == 0 ? 0u : (ax == 1 ? n0 : n01))];
        const double h = axis_h(g, ax);
        int i, j, k;
        node_of(g, c, i, j, k);
        const AxisLine L = axis_line(g, i, j, k, ax);
        const double dist = eno2_fore_distance(f, L, h);
        d.p[2 * ax][c] = (T)dist;
        d.p[2 * ax + 1][c + L.stride] = (T)(h - dist);
    }
}

// one node of an ENORK2 reinitialization stage, all reads from global memory (clamped)
template <typename T>
__device__ __forceinline__ void enork2_reinit_node(const T *__restrict__ phi_s, const T *__restrict__ phi_n,
                                                   T *__restrict__ out, const uint8_t *__restrict__ flags,
                                                   const Ptr6<const T> &d, const Grid &g, int stage, int i, int j,
                                                   int k)
{
    const long long c = node_index(g, i, j, k);
    const uint8_t fl = __ldg(flags + c);
    const T hs[3] = {(T)g.dx, (T)g.dy, (T)g.dz};
    T df[3], db[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        T p[7];
        load_line7(phi_s, axis_line(g, i, j, k, ax), p);
        eno2_pair(p, flagged_distance(fl, 2 * ax, d, c, hs[ax]), flagged_distance(fl, 2 * ax + 1, d, c, hs[ax]),
                  hs[ax], T(0), T(0), df[ax], db[ax]);
    }
    const bool neg = fl & MASK_BIT;
    const T gn = godunov_norm(neg, df[0], db[0], df[1], db[1], df[2], db[2]);
    const T step = (gn - T(1)) * pseudo_dt(fl, d, c, hs[0], hs[1], hs[2]) * (neg ? T(-1) : T(1));
    const T pn = stage == 0 ? T(0) : __ldg(phi_n + c);
    out[c] = rk2_combine(stage, pn, __ldg(phi_s + c), step);
}

template <typename T>
__global__ void __launch_bounds__(BX *BY) k_enork2_reinit_stage(const T *__restrict__ phi_s,
                                                                  const T *__restrict__ phi_n, T *__restrict__ out,
                                                                  const uint8_t *__restrict__ flags, Ptr6<const T> d,
                                                                  Grid g, int stage)
{
    int i, j, k;
    if (!fused_node(g, i, j, k)) return;
    enork2_reinit_node<T>(phi_s, phi_n, out, flags, d, g, stage, i, j, k);
}

// v = sign(F) * n / max(|n|, floor) with the ENO upwind normal (enork2_extend.cu:103-141,
// ENORK2Extend.m:26-42)
template <typename T>
__global__ void __launch_bounds__(BX *BY) k_enork2_velocity(const T *__restrict__ phi, Ptr6<const T> d, Ptr3<T> v,
                                                              Grid g, T floor)
{
    int i, j, k;
    if (!fused_node(g, i, j, k)) return;
    const long long c = node_index(g, i, j, k);
    T n[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        T p[7];
        load_line7(phi, axis_line(g, i, j, k, ax), p);
        n[ax] = eno2_upwind(p, __ldg(d.p[2 * ax] + c), __ldg(d.p[2 * ax + 1] + c), (T)axis_h(g, ax));
    }
    const T grad = vmax(sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]), floor);
    const T f0 = __ldg(phi + c);
    const T s = f0 > T(0) ? T(1) : (f0 < T(0) ? T(-1) : T(0));
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) v.p[ax][c] = s * (n[ax] / grad);
}

// quadratic crossing values (enork2_extend.cu:144-211) at the listed nodes
template <typename T>
__global__ void __launch_bounds__(128) k_enork2_crossing(const T *__restrict__ cfield, Ptr6<const T> d, Ptr6<T> cp,
                                                           NodeList list, Grid g)
{
    const unsigned n = *list.count;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const long long c = list.idx[t];
        int i, j, k;
        node_of(g, c, i, j, k);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            T p[7], cf, cb;
            load_line7(cfield, axis_line(g, i, j, k, ax), p);
            eno2_crossing(p, __ldg(d.p[2 * ax] + c), __ldg(d.p[2 * ax + 1] + c), (T)axis_h(g, ax), cf, cb);
            cp.p[2 * ax][c] = cf;
            cp.p[2 * ax + 1][c] = cb;
        }
    }
}

// one node of an ENORK2 extension stage, all reads from global memory (clamped)
template <typename T>
__device__ __forceinline__ void enork2_extend_node(const T *__restrict__ c_s, const T *__restrict__ c_n,
                                                   T *__restrict__ out, const uint8_t *__restrict__ flags,
                                                   const Ptr6<const T> &d, const Ptr6<const T> &cp,
                                                   const Ptr3<const T> &v, const Grid &g, int stage, int i, int j, int k)
{
    const long long c = node_index(g, i, j, k);
    const uint8_t fl = __ldg(flags + c);
    const T hs[3] = {(T)g.dx, (T)g.dy, (T)g.dz};
    T df[3], db[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        T p[7];
        load_line7(c_s, axis_line(g, i, j, k, ax), p);
        const bool ff = fl & (1u << (2 * ax)), fb = fl & (1u << (2 * ax + 1));
        eno2_pair(p, ff ? __ldg(d.p[2 * ax] + c) : hs[ax], fb ? __ldg(d.p[2 * ax + 1] + c) : hs[ax], hs[ax],
                  ff ? __ldg(cp.p[2 * ax] + c) : T(0), fb ? __ldg(cp.p[2 * ax + 1] + c) : T(0), df[ax], db[ax]);
    }
    const T step = upwind_dot(__ldg(v.p[0] + c), __ldg(v.p[1] + c), __ldg(v.p[2] + c), df[0], db[0], df[1], db[1],
                              df[2], db[2]) *
                   pseudo_dt(fl, d, c, hs[0], hs[1], hs[2]);
    const T pn = stage == 0 ? T(0) : __ldg(c_n + c);
    out[c] = rk2_combine(stage, pn, __ldg(c_s + c), step);
}

template <typename T>
__global__ void __launch_bounds__(BX *BY) k_enork2_extend_stage(const T *__restrict__ c_s, const T *__restrict__ c_n,
                                                                  T *__restrict__ out, const uint8_t *__restrict__ flags,
                                                                  Ptr6<const T> d, Ptr6<const T> cp, Ptr3<const T> v,
                                                                  Grid g, int stage)
{
    int i, j, k;
    if (!fused_node(g, i, j, k)) return;
    enork2_extend_node<T>(c_s, c_n, out, flags, d, cp, v, g, stage, i, j, k);
}

}  // namespace

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------

inline int list_blocks()
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

template <typename T>
cudaError_t launch_set_distance(const T *phi, Ptr6<T> dist, const Grid &g, bool quintic, EdgeLists e, cudaStream_t s)
{
    cudaError_t err = cudaMemsetAsync(e.count, 0, 3 * sizeof(unsigned), s);
    if (err != cudaSuccess) return err;
    k_dist_scan<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi, dist, e, g);
    if (quintic)
        k_dist_roots<T, true><<<list_blocks() * 4, 128, 0, s>>>(phi, dist, e, g);
    else
        k_dist_roots<T, false><<<list_blocks() * 4, 128, 0, s>>>(phi, dist, e, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_classify(const T *phi0, Ptr6<const T> dist, uint8_t *flags, NodeList list, const Grid &g,
                            cudaStream_t s)
{
    if (list.idx) {
        cudaError_t err = cudaMemsetAsync(list.count, 0, sizeof(unsigned), s);
        if (err != cudaSuccess) return err;
    }
    if constexpr (std::is_same<T, float>::value) {
        auto aligned = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
        bool vec = g.num % 4 == 0 && aligned(phi0) && aligned(flags);
        for (int q = 0; q < 6; ++q) vec = vec && aligned(dist.p[q]);
        if (vec) {
            const long long n4 = g.num / 4;
            k_classify4<<<(unsigned)((n4 + 255) / 256), 256, 0, s>>>(phi0, dist, flags, list, n4, (float)g.dx,
                                                                   (float)g.dy, (float)g.dz, (float)(1e-6 * g.dx));
            return cudaGetLastError();
        }
    }
    k_classify<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi0, dist, flags, list, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reinit_stage(const T *phi_s, const T *phi_n, T *out, const uint8_t *flags, Ptr6<const T> dist,
                                const Grid &g, int stage, bool eno3, bool fast, cudaStream_t s)
{
    dim3 gr = node_grid(g), bl(BX, BY);
    if (eno3) {
        if (fast)
            k_reinit_stage<T, true, true><<<gr, bl, 0, s>>>(phi_s, phi_n, out, flags, dist, g, stage);
        else
            k_reinit_stage<T, true, false><<<gr, bl, 0, s>>>(phi_s, phi_n, out, flags, dist, g, stage);
    } else {
        if (fast)
            k_reinit_stage<T, false, true><<<gr, bl, 0, s>>>(phi_s, phi_n, out, flags, dist, g, stage);
        else
            k_reinit_stage<T, false, false><<<gr, bl, 0, s>>>(phi_s, phi_n, out, flags, dist, g, stage);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_extension_velocity(const T *phi, const uint8_t *flags, Ptr6<const T> dist, Ptr3<T> v, const Grid &g,
                                      bool eno3, double floor, NodeList flagged, cudaStream_t s)
{
    if constexpr (std::is_same<T, float>::value) {
        if (flagged.idx) {
            cudaError_t err = launch_velocity_tiled(phi, flags, v, g, (float)floor, s);
            if (err != cudaSuccess) return err;
            if (eno3)
                k_velocity_list<true><<<list_blocks(), 128, 0, s>>>(phi, flags, dist, v, flagged, g, (float)floor);
            else
                k_velocity_list<false><<<list_blocks(), 128, 0, s>>>(phi, flags, dist, v, flagged, g, (float)floor);
            return cudaGetLastError();
        }
    }
    if (eno3)
        k_extension_velocity<T, true><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi, flags, dist, v, g, (T)floor);
    else
        k_extension_velocity<T, false><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi, flags, dist, v, g, (T)floor);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_crossing(const T *c, Ptr6<const T> dist, Ptr6<T> cp, NodeList list, const Grid &g, bool cubic,
                            cudaStream_t s)
{
    if (cubic)
        k_crossing<T, true><<<list_blocks(), 128, 0, s>>>(c, dist, cp, list, g);
    else
        k_crossing<T, false><<<list_blocks(), 128, 0, s>>>(c, dist, cp, list, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_extend_stage(const T *c_s, const T *c_n, T *out, const uint8_t *flags, Ptr6<const T> dist,
                                Ptr6<const T> cp, Ptr3<const T> v, const Grid &g, int stage, bool eno3, bool fast,
                                cudaStream_t s)
{
    dim3 gr = node_grid(g), bl(BX, BY);
    if (eno3) {
        if (fast)
            k_extend_stage<T, true, true><<<gr, bl, 0, s>>>(c_s, c_n, out, flags, dist, cp, v, g, stage);
        else
            k_extend_stage<T, true, false><<<gr, bl, 0, s>>>(c_s, c_n, out, flags, dist, cp, v, g, stage);
    } else {
        if (fast)
            k_extend_stage<T, false, true><<<gr, bl, 0, s>>>(c_s, c_n, out, flags, dist, cp, v, g, stage);
        else
            k_extend_stage<T, false, false><<<gr, bl, 0, s>>>(c_s, c_n, out, flags, dist, cp, v, g, stage);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_advect_stage(const T *phi_s, const T *phi_n, T *out, Ptr3<const T> v, const T *speed,
                                const double *dt, const Grid &g, int stage, bool fast, cudaStream_t s)
{
    if (fast)
        k_advect_stage<T, true><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi_s, phi_n, out, v, speed, dt, g, stage);
    else
        k_advect_stage<T, false><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi_s, phi_n, out, v, speed, dt, g, stage);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_set_distance_eno2(const T *phi, Ptr6<T> dist, const Grid &g, EdgeLists e, cudaStream_t s)
{
    cudaError_t err = cudaMemsetAsync(e.count, 0, 3 * sizeof(unsigned), s);
    if (err != cudaSuccess) return err;
    k_dist_scan<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi, dist, e, g);
    k_dist_roots_eno2<T><<<list_blocks() * 4, 128, 0, s>>>(phi, dist, e, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_enork2_reinit_stage(const T *phi_s, const T *phi_n, T *out, const uint8_t *flags,
                                       Ptr6<const T> dist, const Grid &g, int stage, cudaStream_t s)
{
    k_enork2_reinit_stage<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi_s, phi_n, out, flags, dist, g, stage);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_enork2_velocity(const T *phi, Ptr6<const T> dist, Ptr3<T> v, const Grid &g, double floor,
                                   cudaStream_t s)
{
    k_enork2_velocity<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi, dist, v, g, (T)floor);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_enork2_crossing(const T *c, Ptr6<const T> dist, Ptr6<T> cp, NodeList list, const Grid &g,
                                   cudaStream_t s)
{
    k_enork2_crossing<T><<<list_blocks(), 128, 0, s>>>(c, dist, cp, list, g);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_enork2_extend_stage(const T *c_s, const T *c_n, T *out, const uint8_t *flags, Ptr6<const T> dist,
                                       Ptr6<const T> cp, Ptr3<const T> v, const Grid &g, int stage, cudaStream_t s)
{
    k_enork2_extend_stage<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(c_s, c_n, out, flags, dist, cp, v, g, stage);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reinit_residual(const T *phi, const uint8_t *flags, Ptr6<const T> dist, const Grid &g, double band,
                                   const ResidualState &st, cudaStream_t s)
{
    k_reinit_residual<T><<<node_grid(g), dim3(BX, BY), 0, s>>>(phi, flags, dist, g, band, st);
    return cudaGetLastError();
}

#define VSL_INSTANTIATE_FUSED(T)                                                                                   \
    template cudaError_t launch_set_distance<T>(const T *, Ptr6<T>, const Grid &, bool, EdgeLists, cudaStream_t);   \
    template cudaError_t launch_classify<T>(const T *, Ptr6<const T>, uint8_t *, NodeList, const Grid &,            \
                                            cudaStream_t);                                                          \
    template cudaError_t launch_reinit_stage<T>(const T *, const T *, T *, const uint8_t *, Ptr6<const T>,          \
                                                const Grid &, int, bool, bool, cudaStream_t);                       \
    template cudaError_t launch_extension_velocity<T>(const T *, const uint8_t *, Ptr6<const T>, Ptr3<T>,           \
                                                      const Grid &, bool, double, NodeList, cudaStream_t);          \
    template cudaError_t launch_reinit_residual<T>(const T *, const uint8_t *, Ptr6<const T>, const Grid &, double, \
                                                   const ResidualState &, cudaStream_t);                           \
    template cudaError_t launch_crossing<T>(const T *, Ptr6<const T>, Ptr6<T>, NodeList, const Grid &, bool,        \
                                            cudaStream_t);                                                          \
    template cudaError_t launch_extend_stage<T>(const T *, const T *, T *, const uint8_t *, Ptr6<const T>,          \
                                                Ptr6<const T>, Ptr3<const T>, const Grid &, int, bool, bool,        \
                                                cudaStream_t);                                                      \
    template cudaError_t launch_advect_stage<T>(const T *, const T *, T *, Ptr3<const T>, const T *,                \
                                                const double *, const Grid &, int, bool, cudaStream_t);             \
    template cudaError_t launch_set_distance_eno2<T>(const T *, Ptr6<T>, const Grid &, EdgeLists, cudaStream_t);    \
    template cudaError_t launch_enork2_reinit_stage<T>(const T *, const T *, T *, const uint8_t *, Ptr6<const T>,   \
                                                       const Grid &, int, cudaStream_t);                            \
    template cudaError_t launch_enork2_velocity<T>(const T *, Ptr6<const T>, Ptr3<T>, const Grid &, double,         \
                                                   cudaStream_t);                                                   \
    template cudaError_t launch_enork2_crossing<T>(const T *, Ptr6<const T>, Ptr6<T>, NodeList, const Grid &,       \
                                                   cudaStream_t);                                                   \
    template cudaError_t launch_enork2_extend_stage<T>(const T *, const T *, T *, const uint8_t *, Ptr6<const T>,   \
                                                       Ptr6<const T>, Ptr3<const T>, const Grid &, int, cudaStream_t);

}  // namespace vsl
