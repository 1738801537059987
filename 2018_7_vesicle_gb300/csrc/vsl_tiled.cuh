// vsl_tiled.cuh -- 2.5D-tiled stage kernels of the mixed-precision (FP32) form.
//
// A block of 32 x 8 threads owns a tile of 32 rows x 8 columns and marches KZ pages along
// z.  The x and y stencils of page k come from a ring of 5 shared-memory planes holding
// the tile with a 3-node halo (clamped at the grid edge when loaded, so the stencil reads
// need no clamping); the z stencil comes from a 7-deep register queue per thread.  One
// barrier per page: at page k the block issues the loads of page k+4 into registers,
// computes page k, then stores page k+4 into the slot page k-1 vacated; the centre of
// page k+3 enters the queue.  In z, the smoothness weights of the window of page k+1 serve
// both the forward derivative at k and the backward derivative at k+1.
//
// Nodes whose update needs the interface-aware (nonuniform) stencil -- the "band" -- are
// not computed by the tile code; the generic per-node code updates them, so the uniform
// WENO5 path runs without divergence.  For the reinitialization a node is band when the
// sign of phi changes on one of its stencil edges (the reference's trigger); the tiled
// kernel queues those (warp-aggregated atomics) and k_band_stage follows it.  For the
// extension a node is band when one of its distances differs from the spacing (a superset
// of the reference's trigger r1 < h || l1 < h; the band code applies the exact test): a
// static list, which band blocks of the tiled launch itself update.
#pragma once

#include <algorithm>
#include <atomic>
#include <cudaTypedefs.h>
#include <mutex>

#include "vsl_fused.cuh"
#include "vsl_tma.cuh"

namespace vsl {
namespace {

// Pages per block (a launch parameter: the default below, or the value the tuning table
// holds for the grid shape and stage kind) and the occupancy target (compile time).
// Measured on GB300 at 256^3, vesicle step as a graph: 4 blocks per SM (64 registers) beat
// 5 (48 registers with spills) at 16/32/64 pages; with the page loop unrolled by the ring
// length, 10/15/16/20/25/30/32/40 pages gave 33.6/33.0/33.1/32.7/32.4/32.8/33.0/32.9 ms.
#ifndef VSL_TILED_KZ
#define VSL_TILED_KZ 20
#endif
#ifndef VSL_TILED_MIN_BLOCKS
#define VSL_TILED_MIN_BLOCKS 4
#endif
constexpr int TY = 32;  // rows per tile (threadIdx.x)
constexpr int TX = 8;   // columns per tile (threadIdx.y)
constexpr int HALO = 3;
constexpr int SW = TY + 2 * HALO;  // smem row extent (fastest)
constexpr int SH = TX + 2 * HALO;
constexpr int PLANE = SW * SH;
constexpr int RING = 5;

// SK_ENO2 / SK_ENO2R: the ENORK2 extension / reinitialization (quadratic ENO derivatives,
// Heun RK2 stages); SK_VELOCITY: the extension velocity of the nodes without a distance
// flag (a single pass writing three fields, not an RK stage)
enum StageKind { SK_REINIT = 0, SK_EXTEND = 1, SK_ADVECT = 2, SK_ENO2 = 3, SK_ENO2R = 4, SK_VELOCITY = 5 };
// kinds on the WENO5 stencils (their z window weights are carried from page to page)
__host__ __device__ constexpr bool weno_kind(int kind) { return kind <= SK_ADVECT; }
// kinds whose band is the static list of flagged nodes (the band kernel runs beside them)
__host__ __device__ constexpr bool static_band_kind(int kind)
{
    return kind == SK_EXTEND || kind == SK_ENO2 || kind == SK_ENO2R;
}

struct TiledArgs {
    const float *phi_s;
    const float *phi_n;
    float *out;
    const uint8_t *flags;
    Ptr6<const float> d;
    Ptr3<const float> v;
    const float *speed;
    const double *dt;
    unsigned *queue;
    unsigned *counter;
    Grid g;
    int stage;
    float h[3], inv_h[3], eps2[3];
    float dt_uniform;  // 0.3 * min spacing: the pseudo time step of a node with no crossing
    int kz;            // pages per block
    Ptr3<float> w;     // SK_VELOCITY: the velocity written
    float floor;       // SK_VELOCITY: the floor of |grad phi|
    BandShadow sh;     // static-band kinds: the FP64 shadows and crossing values of the band
    int band_z;        // static-band kinds: page slabs of band blocks after the tile blocks
    int eno3;          // the extension's band takes the ENO3 (WENORK3) interface scheme
};

constexpr int PER_THREAD = (PLANE + TY * TX - 1) / (TY * TX);  // halo elements per thread
// cells of a TMA ring slot per thread (the fix-up of an edge tile's halo)
constexpr int TMA_FIX = (TMA_BOX_ROWS * TMA_BOX_COLS + TY * TX - 1) / (TY * TX);

// a ring slot known at compile time (the unrolled page loop)
template <int N> struct RingSlot {
    __host__ __device__ constexpr operator int() const { return N; }
};

// Upwind quadratic-ENO derivative of a line with no crossing (eno2_pair with r1 = l1 = h:
// (v2 - v0)/h - h * minmod/2h^2 forward, (v0 - v1)/h + h * minmod/2h^2 backward, folded
// into one product with 1/h); back selects the backward one (speed > 0).
__device__ __forceinline__ float eno2_upwind_uniform(const float p[7], bool back, float inv_h)
{
    const float v1 = p[2], v0 = p[3], v2 = p[4];
    const float p2 = v1 - 2.f * v0 + v2;
    if (back) return (v0 - v1 + 0.5f * minmod(p2, v0 - 2.f * v1 + p[1])) * inv_h;
    return (v2 - v0 - 0.5f * minmod(p2, v0 - 2.f * v2 + p[5])) * inv_h;
}

// both quadratic-ENO derivatives of a line with no crossing
__device__ __forceinline__ void eno2_pair_uniform(const float p[7], float inv_h, float &fore, float &back)
{
    const float v1 = p[2], v0 = p[3], v2 = p[4];
    const float p2 = v1 - 2.f * v0 + v2;
    fore = (v2 - v0 - 0.5f * minmod(p2, v0 - 2.f * v2 + p[5])) * inv_h;
    back = (v0 - v1 + 0.5f * minmod(p2, v0 - 2.f * v1 + p[1])) * inv_h;
}

// One tile of one stage: the TY x TX block's tile (bx, by) marching pages bz * kz ..
// (bz + 1) * kz - 1 of the grid of `a` (the work of one block of k_stage_tiled, or of one
// work item of the batched kernel).  smem: the block's plane ring.
//
// Planes reach the ring in one of two ways.  Without TMA every thread loads its share of a
// plane (clamped halo) into registers one page ahead and stores it after the page's reads.
// With TMA thread 0 issues one tensor copy per plane, which completes on the slot's
// mbarrier; thread 0 waits for page k+3 before the barrier of page k, which passes the
// landed plane on to the other threads.  A slot's plane is then
// TMA_BOX_ROWS wide, its first row 4 rows below the tile (the copy's innermost coordinate
// is a multiple of 16 bytes).  A copy reads zeros outside the grid; on tiles at the grid's
// edge each thread then gives its (at most three) cells outside the grid the value of the
// nearest cell inside, the clamped halo of the register path, so both paths see the same
// planes.
template <int KIND, int STAGE, bool TMA = false>
__device__ __forceinline__ void stage_tile(const TiledArgs &a, float *smem, int bx, int by, int bz,
                                           const CUtensorMap *tm = nullptr, uint64_t *bars = nullptr,
                                           unsigned *fixtab = nullptr)
{
    constexpr int PITCH = TMA ? TMA_BOX_ROWS : SW;  // ring row extent (rows of the grid)
    constexpr int PSTR = TMA ? TMA_SLOT_FLOATS : PLANE;  // floats per ring slot
    constexpr int XO = TMA ? 4 : HALO;  // ring index of the tile's first row
    // ring slot sl, tile column jj (0 .. SH-1, halo included), ring row ii
    auto S = [smem](int sl, int jj, int ii) -> float & { return smem[sl * PSTR + jj * PITCH + ii]; };
    const Grid &g = a.g;
    // the launch is always TY x TX threads: the first two elements of every thread's share
    // of a plane are then in the plane without a test
    __builtin_assume(threadIdx.x < TY);
    __builtin_assume(threadIdx.y < TX);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * TY + tx;
    const int i0 = bx * TY, j0 = by * TX;
    const int i = i0 + tx, j = j0 + ty;
    const int k0 = bz * a.kz;
    const int k1 = min(k0 + a.kz, g.pges);
    const bool active = i < g.rows && j < g.cols;
    // ring slot of page p (p >= k0): counted from the block's first page, so that in the
    // loop unrolled by RING the slots are compile-time constants
    auto slot = [k0](int p) { return (p - k0) % RING; };

    // this thread's share of a tile plane (with halo): smem index and in-page offset of up
    // to PER_THREAD elements; the same for every page, only the page base changes
    // element tid + r*TY*TX of the plane; offsets are within one page (< 2^31)
    int e_off[PER_THREAD];
    if constexpr (!TMA) {
#pragma unroll
        for (int r = 0; r < PER_THREAD; ++r) {
            const int e = tid + r * TY * TX;
            const int sy = e / SW, sx = e - sy * SW;
            e_off[r] = clampi(j0 + sy - HALO, g.cols) * g.rows + clampi(i0 + sx - HALO, g.rows);
        }
    }
    // node offsets fit in 32 bits (grids hold at most 2^31 - 1 nodes), so an address is the
    // base pointer plus one widened 32-bit offset
    const unsigned plane = (unsigned)g.plane;
    // pages are fetched at p >= k0 >= 0: only the top edge clamps
    auto page_base = [&](int p) { return a.phi_s + (unsigned)min(p, g.pges - 1) * plane; };
    float pre[PER_THREAD];
    auto fetch = [&](int p) {
        const float *src = page_base(p);
#pragma unroll
        for (int r = 0; r < PER_THREAD; ++r)
            if (tid + r * TY * TX < PLANE) pre[r] = __ldg(src + e_off[r]);
    };
    auto store_slot = [&](int sl) {
        float *dst = &S(sl, 0, 0);
#pragma unroll
        for (int r = 0; r < PER_THREAD; ++r)
            if (tid + r * TY * TX < PLANE) dst[tid + r * TY * TX] = pre[r];
    };
    // TMA: the copy of page p into slot sl and the wait for a slot's next fill (thread 0); a
    // slot's n-th fill completes phase n of its barrier (ph: the parity each slot waits for).
    // A wait that gave up (a copy that never completed) is counted and thread 0 waits for no
    // later copy, so that the block ends in bounded time on stale planes.
    unsigned ph = 0u;
    bool gave_up = false;
    // edge tiles: fixtab[r][tid] = this thread's cell e = tid + r*TY*TX of a slot when it lies
    // outside the grid, as (e << 16) | (offset of the clamped cell) + 1, else 0 (in shared
    // memory: no registers held through the page loop)
    const bool edge =
        TMA && !(i0 >= XO && i0 + TY + HALO <= g.rows && j0 >= HALO && j0 + TX + HALO <= g.cols);
    if constexpr (TMA) {
        if (edge) {
#pragma unroll
            for (int r = 0; r < TMA_FIX; ++r) {
                unsigned f = 0u;
                const int e = tid + r * TY * TX;
                if (e < TMA_BOX_ROWS * TMA_BOX_COLS) {
                    const int jj = e / TMA_BOX_ROWS, ii = e - jj * TMA_BOX_ROWS;
                    const int gj = j0 - HALO + jj, gi = i0 - XO + ii;
                    if (gj < 0 || gj >= g.cols || gi < 0 || gi >= g.rows) {
                        const int src =
                            (clampi(gj, g.cols) - j0 + HALO) * TMA_BOX_ROWS + clampi(gi, g.rows) - i0 + XO;
                        f = ((unsigned)e << 16) | (unsigned)(src + 1);
                    }
                }
                fixtab[r * TY * TX + tid] = f;
            }
        }
    }
    // after the copy of slot sl has landed: the cells outside the grid (each thread its own
    // entries, so no barrier), then the proxy fence that orders these writes before a later
    // copy into the slot
    auto fix_slot = [&](int sl) {
        if constexpr (TMA) {
            if (edge) {
                float *pl = &S(sl, 0, 0);
#pragma unroll
                for (int r = 0; r < TMA_FIX; ++r) {
                    const unsigned f = fixtab[r * TY * TX + tid];
                    if (f) pl[f >> 16] = pl[(f & 0xFFFFu) - 1u];
                }
                fence_proxy_async();
            }
        }
    };
    auto tma_fetch = [&](int p, int sl) {
        mbar_expect_tx(&bars[sl], TMA_PLANE_BYTES);
        tma_load_box(&S(sl, 0, 0), tm, i0 - XO, j0 - HALO, min(p, g.pges - 1), &bars[sl]);
    };
    auto tma_wait = [&](int sl) {
        if (!gave_up) gave_up = !mbar_wait(&bars[sl], (ph >> sl) & 1u);
        ph ^= 1u << sl;
    };

    float q[7];  // phi_s(i, j, k-3 .. k+3)
    if constexpr (TMA) {
        // pages k0 .. k0+3 (k1 > k0, so all of them are read); thread 0 alone waits for a
        // copy, and the block barrier after its wait passes the plane on to the other threads
        if (tid == 0) {
            for (int p = k0; p < k0 + 4; ++p) tma_fetch(p, slot(p));
            for (int p = k0; p < k0 + 3; ++p) tma_wait(slot(p));
        }
    } else {
        for (int p = k0; p < k0 + 4; ++p) {
            fetch(p);
            store_slot(slot(p));
        }
    }
    {
        const int ic = clampi(i, g.rows), jc = clampi(j, g.cols);
        const unsigned col = (unsigned)jc * (unsigned)g.rows + (unsigned)ic;
#pragma unroll
        for (int s = 0; s < 3; ++s) q[s] = __ldg(a.phi_s + (col + (unsigned)clampi(k0 - 3 + s, g.pges) * plane));
    }
    __syncthreads();
    if constexpr (TMA) {
        // the halo cells outside the grid; an active node's own cell is never one of them, and
        // the barrier of page k0 orders these writes before the stencil reads
        for (int p = k0; p < k0 + 3; ++p) fix_slot(slot(p));
    }
#pragma unroll
    for (int s = 3; s < 6; ++s) q[s] = S(slot(k0 + s - 3), ty + HALO, tx + XO);
    // reciprocal smoothness weights of the z window of page k0 (backward derivative)
    float zr1 = 0.f, zr2 = 0.f, zr3 = 0.f;
    if constexpr (weno_kind(KIND))
        weno5_window_weights(q[1] - q[0], q[2] - q[1], q[3] - q[2], q[4] - q[3], q[5] - q[4], a.eps2[2], zr1, zr2,
                             zr3);

    const unsigned lane = tid & 31;
    // the advection's time step (formed on the device by an earlier launch): read once
    const float dt_adv = KIND == SK_ADVECT ? (float)__ldg(a.dt) : 0.f;
    // per-node inputs of the next page, loaded one page ahead
    const unsigned col_base = (unsigned)clampi(j, g.cols) * (unsigned)g.rows + (unsigned)clampi(i, g.rows);
    unsigned c = col_base + (unsigned)k0 * plane;
    uint8_t fl_next = 0;
    float pn_next = 0.f, v0_next = 0.f, v1_next = 0.f, v2_next = 0.f, sp_next = 1.f;
    auto load_node = [&](unsigned cc) {
        if (KIND != SK_ADVECT) fl_next = __ldg(a.flags + cc);
        if (STAGE != 0) pn_next = __ldg(a.phi_n + cc);
        if (KIND == SK_EXTEND || KIND == SK_ADVECT || KIND == SK_ENO2) {
            v0_next = __ldg(a.v.p[0] + cc);
            v1_next = __ldg(a.v.p[1] + cc);
            v2_next = __ldg(a.v.p[2] + cc);
            if (KIND == SK_ADVECT && a.speed) sp_next = __ldg(a.speed + cc);
        }
    };
    if (active && k0 < k1) load_node(c);
    // one page: the slots of pages k, k+3 and k+4 (= k-1) are RingSlot constants in the
    // unrolled loop and plain ints in the remainder
    auto page = [&](auto sk, auto sk3, auto sk4, int k) {
        // every warp has finished page k-1 and stored page k+3 (TMA: thread 0 has seen the
        // copy of page k+3 land)
        if constexpr (TMA) {
            if (tid == 0) tma_wait(int(sk3));
        }
        __syncthreads();
        if constexpr (TMA) {
            // page k+4 into the slot of page k-1; pages past k1+2 are never read
            if (tid == 0 && k + 4 <= k1 + 2) {
                fence_proxy_async();
                tma_fetch(k + 4, int(sk4));
            }
            fix_slot(int(sk3));  // page k+3, read as a stencil plane three barriers later
        }
        q[6] = S(int(sk3), ty + HALO, tx + XO);
        if constexpr (!TMA) fetch(k + 4);  // loads in flight during this page's arithmetic, stored at its end
        const float *P = &S(int(sk), 0, 0);
        const uint8_t fl = fl_next;
        const float pn = pn_next, vx0 = v0_next, vy0 = v1_next, vz0 = v2_next, sp = sp_next;
        if (active && k + 1 < k1) load_node(c + plane);

        // z window of page k+1: its weights give the forward derivative here and the
        // backward derivative at the next page
        const float v1 = q[1] - q[0], v2 = q[2] - q[1], v3 = q[3] - q[2], v4 = q[4] - q[3], v5 = q[5] - q[4],
                    v6 = q[6] - q[5];
        float nr1 = 0.f, nr2 = 0.f, nr3 = 0.f;
        if constexpr (weno_kind(KIND)) weno5_window_weights(v2, v3, v4, v5, v6, a.eps2[2], nr1, nr2, nr3);

        bool band = false;
        if (active) {
            float px[7], py[7];
#pragma unroll
            for (int s = 0; s < 7; ++s) {
                px[s] = P[(ty + s) * PITCH + tx + XO];
                py[s] = P[(ty + HALO) * PITCH + tx + XO - HALO + s];
            }
            const float ps = q[3];
            float step = 0.f;
            bool compute = true;
            if (KIND != SK_ADVECT && KIND != SK_VELOCITY && (fl & FIXED_BIT)) compute = false;
            if (compute && KIND == SK_REINIT) {
                band = px[2] * px[3] < 0.f || px[3] * px[4] < 0.f || py[2] * py[3] < 0.f || py[3] * py[4] < 0.f ||
                       q[2] * q[3] < 0.f || q[3] * q[4] < 0.f;
            } else if (static_band_kind(KIND) || KIND == SK_VELOCITY) {
                // every node of the static list (fixed ones too) belongs to the band kernel,
                // which may run at the same time: each node has exactly one writer
                band = (fl & 0x3F) != 0;
            }
            if (compute && !band && KIND == SK_REINIT) {
                // the Godunov norm needs both one-sided derivatives of every axis
                float dxf, dxb, dyf, dyb;
                weno5_pair_fast2(px, a.inv_h[0], a.eps2[0], dxf, dxb);
                weno5_pair_fast2(py, a.inv_h[1], a.eps2[1], dyf, dyb);
                // z: backward window of page k (weights carried), forward = reversed window of k+1
                float2 q1, q2, q3;
                weno5_candidates2(f2(v1, v6), f2(v2, v5), f2(v3, v4), f2(v4, v3), f2(v5, v2), q1, q2, q3);
                const float2 dz = mul2(weno5_combine2(q1, q2, q3, f2(zr1, nr3), f2(zr2, nr2), f2(zr3, nr1)),
                                       f2s(a.inv_h[2]));
                const bool neg = fl & MASK_BIT;
                const float dtn = (fl & 0x3F) ? pseudo_dt(fl, a.d, (long long)c, a.h[0], a.h[1], a.h[2]) : a.dt_uniform;
                const float gn = godunov_norm(neg, dxf, dxb, dyf, dyb, dz.y, dz.x);
                step = (gn - 1.f) * dtn * (neg ? -1.f : 1.f);
            } else if (compute && !band && KIND == SK_ENO2R) {
                // ENORK2 reinitialization: Godunov norm of both quadratic-ENO derivatives
                float xf, xb, yf, yb, zf, zb;
                eno2_pair_uniform(px, a.inv_h[0], xf, xb);
                eno2_pair_uniform(py, a.inv_h[1], yf, yb);
                eno2_pair_uniform(q, a.inv_h[2], zf, zb);
                const bool neg = fl & MASK_BIT;
                const float gn = godunov_norm(neg, xf, xb, yf, yb, zf, zb);
                step = (gn - 1.f) * a.dt_uniform * (neg ? -1.f : 1.f);
            } else if (compute && !band && KIND == SK_ENO2) {
                // ENORK2 extension: the upwind quadratic-ENO derivative of each axis
                const float tr = vx0 * eno2_upwind_uniform(px, vx0 > 0.f, a.inv_h[0]) +
                                 vy0 * eno2_upwind_uniform(py, vy0 > 0.f, a.inv_h[1]) +
                                 vz0 * eno2_upwind_uniform(q, vz0 > 0.f, a.inv_h[2]);
                step = tr * a.dt_uniform;
            } else if (compute && !band && (KIND == SK_EXTEND || KIND == SK_ADVECT)) {
                // transport sum_ax min(0,v) D+ + max(0,v) D-: the velocity is fixed, so each
                // axis needs only its upwind derivative (D- where v > 0); x and y share one
                // packed evaluation, z reuses the carried window weights
                const float ux = KIND == SK_ADVECT ? vx0 * sp : vx0;
                const float uy = KIND == SK_ADVECT ? vy0 * sp : vy0;
                const float uz = KIND == SK_ADVECT ? vz0 * sp : vz0;
                const float2 dxy = weno5_upwind2(px, ux > 0.f, py, uy > 0.f, f2(a.inv_h[0], a.inv_h[1]),
                                                 f2(a.eps2[0], a.eps2[1]));
                const bool zb = uz > 0.f;
                const float dz = weno5_with_weights(zb ? v1 : v6, zb ? v2 : v5, zb ? v3 : v4, zb ? v4 : v3,
                                                    zb ? v5 : v2, zb ? zr1 : nr3, zb ? zr2 : nr2, zb ? zr3 : nr1) *
                                 a.inv_h[2];
                const float tr = ux * dxy.x + uy * dxy.y + uz * dz;
                step = KIND == SK_EXTEND ? tr * a.dt_uniform : dt_adv * tr;
            }
            if (!band && KIND == SK_VELOCITY) {
                // the unit normal of a node away from the interface: each axis reconstructs
                // the side it keeps (D+ where |p4| < |p2|, else D-), x and y as the lanes of
                // one packed WENO5, z with itself in both lanes
                const bool bx = !(fabsf(px[4]) < fabsf(px[2])), by = !(fabsf(py[4]) < fabsf(py[2]));
                const bool bz = !(fabsf(q[4]) < fabsf(q[2]));
                const float2 dxy =
                    weno5_upwind2(px, bx, py, by, f2(a.inv_h[0], a.inv_h[1]), f2(a.eps2[0], a.eps2[1]));
                const float2 dzz = weno5_upwind2(q, bz, q, bz, f2s(a.inv_h[2]), f2s(a.eps2[2]));
                const float n[3] = {dxy.x, dxy.y, dzz.x};
                const float grad = vmax(sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]), a.floor);
                const float sg = ps > 0.f ? 1.f : (ps < 0.f ? -1.f : 0.f);
#pragma unroll
                for (int ax = 0; ax < 3; ++ax) a.w.p[ax][c] = sg * (n[ax] / grad);
            } else if (!band) {
                a.out[c] = (KIND == SK_ENO2 || KIND == SK_ENO2R) ? rk2_combine(STAGE, pn, ps, step)
                                                                  : rk3_combine(STAGE, pn, ps - step);
            }
        }
        if (KIND == SK_REINIT) {  // the extension's band is the static list of flagged nodes
            const unsigned m = __ballot_sync(0xffffffffu, band);
            if (m) {
                unsigned base = 0;
                const int leader = __ffs(m) - 1;
                if ((int)lane == leader) base = atomicAdd(a.counter, (unsigned)__popc(m));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (band) {
                    const unsigned rank = __popc(m & ((1u << lane) - 1u));
                    a.queue[base + rank] = c;
                }
            }
        }
        // page k+4 goes to the slot of page k-1, which no warp reads any more
        if constexpr (!TMA) store_slot(int(sk4));
        zr1 = nr1;
        zr2 = nr2;
        zr3 = nr3;
#pragma unroll
        for (int s = 0; s < 6; ++s) q[s] = q[s + 1];
        c += plane;
    };
    using I0 = RingSlot<0>;
    using I1 = RingSlot<1>;
    using I2 = RingSlot<2>;
    using I3 = RingSlot<3>;
    using I4 = RingSlot<4>;
    static_assert(RING == 5, "the unrolled page loop assumes a ring of 5 planes");
    int k = k0;
    for (; k + RING <= k1; k += RING) {
        page(I0{}, I3{}, I4{}, k);
        page(I1{}, I4{}, I0{}, k + 1);
        page(I2{}, I0{}, I1{}, k + 2);
        page(I3{}, I1{}, I2{}, k + 3);
        page(I4{}, I2{}, I3{}, k + 4);
    }
#pragma unroll 1
    for (int r = 0; k < k1; ++k, ++r) page(r, (r + 3) % RING, (r + 4) % RING, k);
}

// ---------------------------------------------------------------------------------------
// Extension band of the mixed form with FP64 interface data.  Next to a crossing at a
// short distance from a node, the one-sided divided difference between the node (or its
// neighbour) and the crossing value divides the difference of two O(|C|) values by a gap
// of a small fraction of h: in FP32 both values carry an independent rounding of |C| 6e-8,
// which the gap multiplies by h / gap.  The crossing values (computed in FP64 from the FP32
// field) and the flagged nodes' values (kept in FP64 beside the FP32 field, "shadows", and
// updated here) give those differences in FP64; the rest of the stencil arithmetic stays
// FP32 on divided differences of ordinary size.  Nodes off the band (the tiled kernel)
// never form such a difference.
// ---------------------------------------------------------------------------------------

// the stage input at node n next to a crossing: its shadow where n is flagged (every node
// next to a crossing is, unless its own distance rounded to the spacing), else its FP32 value
__device__ __forceinline__ double shadow_or(const BandShadow &sh, const uint8_t *flags, long long n, float v)
{
    return (__ldg(flags + n) & 0x3F) ? __ldg(sh.s_in + n) : (double)v;
}

// one band node of a WENO5 / WENORK3 extension stage (extend_node with the FP64 interface data)
template <bool ENO3>
__device__ __forceinline__ void extend_node_mixed(const TiledArgs &a, const BandShadow &sh, int i, int j, int k)
{
    const Grid &g = a.g;
    const long long c = node_index(g, i, j, k);
    const uint8_t fl = __ldg(a.flags + c);
    const double cs = __ldg(sh.s_in + c);
    float step = 0.f;
    if (!(fl & FIXED_BIT)) {
        float df[3], db[3];
#pragma unroll 1
        for (int ax = 0; ax < 3; ++ax) {
            float p[7];
            const AxisLine L = axis_line(g, i, j, k, ax);
            load_line7(a.phi_s, L, p);
            const float h = a.h[ax];
            const float r1 = flagged_distance(fl, 2 * ax, a.d, c, h);
            const float l1 = flagged_distance(fl, 2 * ax + 1, a.d, c, h);
            if (r1 < h || l1 < h) {
                float rc, lc;
                crossing_gaps(L, ax, a.d, c, r1, l1, h, rc, lc);
                float G[6], pv[7];
                insert_interface_gaps(p, r1, rc, l1, lc, h, 0.f, 0.f, G, pv);
                // The line hs[0..6] in FP64: pv, with the node's shadow cs at 3, and on each
                // side with a crossing the crossing value (2 / 4) and the shadow of the
                // neighbour beyond it (1 / 5).  The differences are taken in FP64 where an
                // end is such a value (the digits cancel there), the quotients in FP32.  A
                // segment between two FP32 values takes the FP32 difference instead: the FP64
                // difference of two FP32 values is exact unless their exponents lie more than
                // 28 apart, and then it lies far from an FP32 rounding boundary, so rounded to
                // FP32 it is the FP32 difference.  Same bits, with 4 of the 6 segments in FP64
                // on a one-sided crossing (FP64 runs at 1/64 of the FP32 rate here).
                const bool rs = r1 < h, both = rs && l1 < h;
                // the side with the crossing (the right one when both have one): the chain
                // e0 .. e4 = hs[2..6] (right) or hs[0..4] (left) and its four segments
                const double cx = __ldg(sh.cp.p[rs ? 2 * ax : 2 * ax + 1] + c);
                const double sn = shadow_or(sh, a.flags, rs ? c + L.stride : c - L.stride, rs ? p[4] : p[2]);
                double e0 = (double)(rs ? pv[2] : pv[0]);
                float x0 = 0.f, x1 = 0.f;  // both sides: segments 0 and 1 in FP64 as well
                if (both) {
                    const double cl = __ldg(sh.cp.p[2 * ax + 1] + c);
                    const double sl = shadow_or(sh, a.flags, c - L.stride, p[2]);
                    x0 = (float)(sl - (double)pv[0]);
                    x1 = (float)(cl - sl);
                    e0 = cl;
                }
                const double e1 = rs ? cs : sn, e3 = rs ? sn : cs, e4 = (double)(rs ? pv[6] : pv[4]);
                const float f0 = (float)(e1 - e0), f1 = (float)(cx - e1), f2 = (float)(e3 - cx),
                            f3 = (float)(e4 - e3);
                // the other side's two segments, between FP32 values
                const float u0 = rs ? pv[0] : pv[4], u1 = rs ? pv[1] : pv[5], u2 = rs ? pv[2] : pv[6];
                const float g0 = __fsub_rn(u1, u0), g1 = __fsub_rn(u2, u1);
                float dd[6] = {rs ? (both ? x0 : g0) : f0, rs ? (both ? x1 : g1) : f1, rs ? f0 : f2,
                               rs ? f1 : f3, rs ? f2 : g0, rs ? f3 : g1};
#pragma unroll
                for (int m = 0; m < 6; ++m) dd[m] = dd[m] / G[m];
                if (ENO3)
                    eno3_nonuniform_pair_dd(G, dd, df[ax], db[ax]);
                else
                    weno_nonuniform_pair_dd(G, dd, df[ax], db[ax]);
            } else {
                weno5_pair_fast(p, a.inv_h[ax], a.eps2[ax], df[ax], db[ax]);
            }
        }
        step = upwind_dot(__ldg(a.v.p[0] + c), __ldg(a.v.p[1] + c), __ldg(a.v.p[2] + c), df[0], db[0], df[1], db[1],
                          df[2], db[2]) *
               pseudo_dt(fl, a.d, c, a.h[0], a.h[1], a.h[2]);
    }
    const double pn = a.stage == 0 ? 0.0 : __ldg(sh.s_n + c);
    const double val = rk3_combine(a.stage, pn, cs - (double)step);
    a.out[c] = (float)val;
    sh.s_out[c] = val;
}

// one band node of an ENORK2 extension stage (enork2_extend_node with the FP64 interface data)
__device__ __forceinline__ void enork2_extend_node_mixed(const TiledArgs &a, const BandShadow &sh, int i, int j, int k)
{
    const Grid &g = a.g;
    const long long c = node_index(g, i, j, k);
    const uint8_t fl = __ldg(a.flags + c);
    const double cs = __ldg(sh.s_in + c);
    float df[3], db[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        float p[7];
        load_line7(a.phi_s, axis_line(g, i, j, k, ax), p);
        const float h = a.h[ax];
        const bool ff = fl & (1u << (2 * ax)), fb = fl & (1u << (2 * ax + 1));
        const float r1 = ff ? __ldg(a.d.p[2 * ax] + c) : h, l1 = fb ? __ldg(a.d.p[2 * ax + 1] + c) : h;
        // eno2_pair: the one-sided differences to a crossing in FP64 (crossing value and shadow)
        const float v4 = p[1], v1 = p[2], v0 = p[3], v2 = p[4], v3 = p[5];
        const float h2 = h * h;
        const float p2 = v1 - 2.f * v0 + v2;
        float p2m = 0.5f * minmod(p2, v0 - 2.f * v2 + v3) / h2;
        const float sr = (r1 == h) ? (v2 - v0) / r1 : (float)(__ldg(sh.cp.p[2 * ax] + c) - cs) / r1;
        df[ax] = sr - r1 * p2m;
        p2m = 0.5f * minmod(p2, v0 - 2.f * v1 + v4) / h2;
        const float sl = (l1 == h) ? (v0 - v1) / l1 : (float)(cs - __ldg(sh.cp.p[2 * ax + 1] + c)) / l1;
        db[ax] = sl + l1 * p2m;
    }
    const float step = upwind_dot(__ldg(a.v.p[0] + c), __ldg(a.v.p[1] + c), __ldg(a.v.p[2] + c), df[0], db[0], df[1],
                                  db[1], df[2], db[2]) *
                       pseudo_dt(fl, a.d, c, a.h[0], a.h[1], a.h[2]);
    const double pn = a.stage == 0 ? 0.0 : __ldg(sh.s_n + c);
    const double val = rk2_combine(a.stage, pn, cs, (double)step);
    a.out[c] = (float)val;
    sh.s_out[c] = val;
}

// one node (offset c) of the static band of a stage of a static-band kind
template <int KIND>
__device__ __forceinline__ void static_band_node(const TiledArgs &a, long long c)
{
    const Grid &g = a.g;
    const int k = (int)(c / g.plane);
    const long long r = c - (long long)k * g.plane;
    const int j = (int)(r / g.rows);
    const int i = (int)(r - (long long)j * g.rows);
    if constexpr (KIND == SK_ENO2)
        enork2_extend_node_mixed(a, a.sh, i, j, k);
    else if constexpr (KIND == SK_ENO2R)
        enork2_reinit_node<float>(a.phi_s, a.phi_n, a.out, a.flags, a.d, g, a.stage, i, j, k);
    else if (a.eno3)
        extend_node_mixed<true>(a, a.sh, i, j, k);
    else
        extend_node_mixed<false>(a, a.sh, i, j, k);
}

// The ENORK2 extension kind, whose uniform path is light, is latency-bound at 4 blocks per SM
// (long-scoreboard stalls, DRAM 35% of peak): 5 blocks (47 registers, no spills) took 100
// pseudo-steps at 256^3 from 26.7 to 23.6 ms.  The ENORK2 reinitialization was slower at 5
// (25.7 -> 27.7 ms) and keeps 4 with the WENO5 kinds.
//
// TMA: the planes by tensor copies (the launch's tensor map of phi_s), else through registers.
//
// Static-band kinds: the last a.band_z page slabs of the launch are band blocks, which
// update the nodes of the classification's flagged list (grid-stride over the list) instead
// of a tile.  They are dispatched after the tile blocks and fill the SMs as tile blocks
// retire, in the same launch; every node still has exactly one writer.
template <int KIND, int STAGE, bool TMA>
__global__ void __launch_bounds__(TY *TX, (KIND == SK_ENO2 ? 5 : VSL_TILED_MIN_BLOCKS))
    k_stage_tiled(const __grid_constant__ TiledArgs a, const __grid_constant__ CUtensorMap tm)
{
    static_assert(SH == TMA_BOX_COLS && PLANE <= TMA_SLOT_FLOATS, "ring layouts");
    if constexpr (static_band_kind(KIND)) {
        const int bz0 = (int)gridDim.z - a.band_z;
        if ((int)blockIdx.z >= bz0) {
            const unsigned nt = TY * TX;
            const unsigned nb = gridDim.x * gridDim.y * (unsigned)a.band_z;
            const unsigned b = ((blockIdx.z - (unsigned)bz0) * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
            const unsigned n = *a.counter;
            for (unsigned t = b * nt + threadIdx.y * TY + threadIdx.x; t < n; t += nb * nt)
                static_band_node<KIND>(a, a.queue[t]);
            return;
        }
    }
    if constexpr (TMA) {
        __shared__ __align__(128) float smem[RING * TMA_SLOT_FLOATS];
        __shared__ __align__(8) uint64_t bars[RING];
        __shared__ unsigned fixtab[TMA_FIX * TY * TX];
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            for (int s = 0; s < RING; ++s) mbar_init(&bars[s], 1);
            mbar_init_fence();
        }
        __syncthreads();
        stage_tile<KIND, STAGE, true>(a, smem, blockIdx.x, blockIdx.y, blockIdx.z, &tm, bars, fixtab);
    } else {
        __shared__ float smem[RING * PLANE];
        stage_tile<KIND, STAGE, false>(a, smem, blockIdx.x, blockIdx.y, blockIdx.z);
    }
}

// Band nodes of one reinitialization stage: the generic per-node update (interface-aware
// stencils), grid-stride over the queue the tiled kernel filled; also clears the other
// stage's counter for its next use.  (The static bands of the other kinds run in band
// blocks of the tiled launch itself, k_stage_tiled.)  No occupancy target (75 registers;
// 8 blocks per SM gained nothing).
template <bool ENO3>
__global__ void __launch_bounds__(128) k_band_stage(TiledArgs a, unsigned *next_counter)
{
    const unsigned n = *a.counter;
    if (next_counter && blockIdx.x == 0 && threadIdx.x == 0) *next_counter = 0u;
    const Grid &g = a.g;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const long long c = a.queue[t];
        const int k = (int)(c / g.plane);
        const long long r = c - (long long)k * g.plane;
        const int j = (int)(r / g.rows);
        const int i = (int)(r - (long long)j * g.rows);
        reinit_node<float, ENO3, true>(a.phi_s, a.phi_n, a.out, a.flags, a.d, g, a.stage, i, j, k);
    }
}

// ---------------------------------------------------------------------------------------
// Batched stages: one launch runs one RK stage of up to BATCH_MAX grids (a batch of
// vesicles).  The work list is every grid's tiles (tile x, tile y, page slab) in order, one
// block per item (the kernel walks the list grid-stride, so a smaller grid of blocks also
// covers it), so small grids that could not fill the GPU alone share its SMs, and a batch
// step issues one launch per stage instead of one per vesicle.
// The stages' order is the launches' order on the stream: no block waits for another.
// Every grid's arguments travel in the kernel parameter (a __grid_constant__ table indexed
// by the block-uniform grid number).
// ---------------------------------------------------------------------------------------
constexpr int BATCH_MAX = TILED_BATCH_MAX;
struct TiledBatch {
    TiledArgs v[BATCH_MAX];
    int start[BATCH_MAX + 1];  // first work item of each grid; start[count] = all items
    int nx[BATCH_MAX], ny[BATCH_MAX];  // tiles along rows and columns
    int tiles[BATCH_MAX];  // tile items of each grid; its band blocks follow them
    int nb[BATCH_MAX];     // static-band kinds: band blocks of each grid
    int count;
};
static_assert(sizeof(TiledBatch) <= 32000, "kernel parameter space");

// the grid of work item w: the last g with start[g] <= w (start is block-uniform)
__device__ __forceinline__ int batch_member(const int *start, int count, int w)
{
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= w)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <int KIND, int STAGE>
__global__ void __launch_bounds__(TY *TX, (KIND == SK_ENO2 ? 5 : VSL_TILED_MIN_BLOCKS))
    k_stage_tiled_batch(const __grid_constant__ TiledBatch B)
{
    __shared__ float smem[RING * PLANE];
    const int total = B.start[B.count];
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int v = batch_member(B.start, B.count, w);
        const int local = w - B.start[v];
        if (local < B.tiles[v]) {
            const int rest = local / B.nx[v];
            stage_tile<KIND, STAGE>(B.v[v], smem, local - rest * B.nx[v], rest % B.ny[v], rest / B.ny[v]);
            __syncthreads();  // the next item's prologue rewrites the plane ring
            continue;
        }
        if constexpr (static_band_kind(KIND)) {
            // band block of grid v: its static band grid-stride, right after its tiles (its
            // planes still in L2)
            const TiledArgs &a = B.v[v];
            const unsigned nt = TY * TX, nb = (unsigned)B.nb[v];
            const unsigned n = *a.counter;
            for (unsigned t = (unsigned)(local - B.tiles[v]) * nt + threadIdx.y * TY + threadIdx.x; t < n; t += nb * nt)
                static_band_node<KIND>(a, a.queue[t]);
        }
    }
}

// The reinitialization's band nodes of one stage of every grid of a batch (k_band_stage per
// grid, all the grids' queued band nodes as one work list in one launch, which follows the
// batched tiled launch that fills the queues).  8 blocks per SM (64 registers): the batch's
// bands are large and latency-bound (64-vesicle batch step 158.0 -> 157.0 ms against 75
// registers).  The static bands of the other kinds run as band blocks of the batched tiled
// launch, each grid's right after its tiles.
struct BandBatch {
    TiledArgs v[BATCH_MAX];     // with each grid's band shadows (static-band kinds)
    unsigned *next[BATCH_MAX];  // reinitialization: the other stage's counter, zeroed here
    int count;
};
static_assert(sizeof(BandBatch) <= 32000, "kernel parameter space");

template <bool ENO3>
__global__ void __launch_bounds__(128, 8) k_band_stage_batch(const __grid_constant__ BandBatch B)
{
    // one work list of every grid's band nodes: the grids' counts, prefix-summed per block,
    // place work item t at node t - first[v] of grid v (first[v] <= t < first[v + 1]), so the
    // blocks share the band nodes of all the grids evenly, whatever the sizes of the bands
    static_assert(BATCH_MAX <= 128, "one counter per thread");
    __shared__ unsigned first[BATCH_MAX + 1];
    if ((int)threadIdx.x < B.count) first[threadIdx.x + 1] = *B.v[threadIdx.x].counter;
    __syncthreads();
    if (threadIdx.x == 0) {
        first[0] = 0u;
        for (int v = 0; v < B.count; ++v) first[v + 1] += first[v];
    }
    __syncthreads();
    // the reinitialization clears the other stage's counters, which this launch does not read
    if (blockIdx.x == 0 && (int)threadIdx.x < B.count && B.next[threadIdx.x]) *B.next[threadIdx.x] = 0u;
    const unsigned total = first[B.count];
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        int lo = 0, hi = B.count - 1;  // the last grid v with first[v] <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (first[mid] <= t)
                lo = mid;
            else
                hi = mid - 1;
        }
        const TiledArgs &a = B.v[lo];
        const Grid &g = a.g;
        const long long c = a.queue[t - first[lo]];
        const int k = (int)(c / g.plane);
        const long long r = c - (long long)k * g.plane;
        const int j = (int)(r / g.rows);
        const int i = (int)(r - (long long)j * g.rows);
        reinit_node<float, ENO3, true>(a.phi_s, a.phi_n, a.out, a.flags, a.d, g, a.stage, i, j, k);
    }
}

}  // namespace

inline TiledArgs tiled_args(const Grid &g)
{
    TiledArgs a{};
    a.g = g;
    const double hh[3] = {g.dx, g.dy, g.dz};
    for (int q = 0; q < 3; ++q) {
        a.h[q] = (float)hh[q];
        a.inv_h[q] = 1.0f / (float)hh[q];
        a.eps2[q] = 1e-6f * (float)hh[q] * (float)hh[q];
    }
    const float hx = (float)g.dx, hy = (float)g.dy, hz = (float)g.dz;
    a.dt_uniform = 0.3f * fminf(fminf(hx, hx), fminf(fminf(hy, hy), fminf(hz, hz)));
    return a;
}

// the band kernels run latency-bound per-node code: 16 blocks of 128 threads per SM
inline int band_blocks() { return list_blocks() * 4; }

// page slabs of band blocks appended to a static-band kind's tile grid gr: as many threads
// as the separate band kernel had (band_blocks() x 128), in blocks of the tile kernel's shape
inline int static_band_slabs(const dim3 &gr)
{
    const long long want = (long long)band_blocks() * 128 / (TY * TX);
    const long long per_slab = (long long)gr.x * gr.y;
    return (int)std::max<long long>(1, (want + per_slab - 1) / per_slab);
}

inline dim3 tiled_grid(const Grid &g, int kz)
{
    return dim3((g.rows + TY - 1) / TY, (g.cols + TX - 1) / TX, (g.pges + kz - 1) / kz);
}

// ---------------------------------------------------------------------------------------
// tuning table: pages per block by grid shape and stage kind (set by an autotuner)
// ---------------------------------------------------------------------------------------
namespace {
struct TileEntry {
    int rows, cols, pges, kind, pages;
};
constexpr int TILE_TABLE = 512;
std::mutex tile_mutex;
TileEntry tile_table[TILE_TABLE];
int tile_count = 0;
}  // namespace

int tile_pages(const Grid &g, int kind)
{
    std::lock_guard<std::mutex> lock(tile_mutex);
    for (int e = 0; e < tile_count; ++e) {
        const TileEntry &t = tile_table[e];
        if (t.rows == g.rows && t.cols == g.cols && t.pges == g.pges && t.kind == kind) return t.pages;
    }
    return VSL_TILED_KZ;
}

int set_tile_pages(int rows, int cols, int pges, int kind, int pages)
{
    if (rows <= 0 || cols <= 0 || pges <= 0) return VSL_ERR_SHAPE;
    if (kind < 0 || kind > 4 || pages < 0 || pages > 65535) return VSL_ERR_VALUE;
    std::lock_guard<std::mutex> lock(tile_mutex);
    for (int e = 0; e < tile_count; ++e) {
        TileEntry &t = tile_table[e];
        if (t.rows == rows && t.cols == cols && t.pges == pges && t.kind == kind) {
            if (pages == 0) {  // back to the default: drop the entry
                t = tile_table[--tile_count];
            } else {
                t.pages = pages;
            }
            return VSL_OK;
        }
    }
    if (pages == 0) return VSL_OK;
    if (tile_count == TILE_TABLE) return VSL_ERR_VALUE;
    tile_table[tile_count++] = TileEntry{rows, cols, pges, kind, pages};
    return VSL_OK;
}


// ---------------------------------------------------------------------------------------
// TMA plane loads: the driver's tensor-map encoder (looked up once through the runtime) and
// the process-wide choice of plane loads (vsl_set_plane_loads)
// ---------------------------------------------------------------------------------------
namespace {
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}
// Register plane loads are the default: measured on GB300 at 256^3, the TMA path ran the
// reinitialization stage in 203 us against 189 us (ncu), 340 against 329 warp instructions
// per node: the stage kernels are issue-bound at the 64-register cap, and the copies' waits,
// the branches of the issuing thread and the edge fix-up cost more issue slots than the
// three loads and three shared stores per node they replace.
#ifndef VSL_PLANE_LOADS
#define VSL_PLANE_LOADS 0
#endif
std::atomic<int> plane_loads{VSL_PLANE_LOADS};  // 1: TMA where the field allows, 0: registers only
}  // namespace

int set_plane_loads(int mode)
{
    if (mode != 0 && mode != 1) return VSL_ERR_VALUE;
    plane_loads.store(mode);
    return VSL_OK;
}
int get_plane_loads() { return plane_loads.load(); }

// bounded TMA waits that gave up since the library was loaded (zero unless a copy failed
// to complete)
cudaError_t tma_timeouts(unsigned *count) { return cudaMemcpyFromSymbol(count, tma_wait_timeouts, sizeof(unsigned)); }

// The tensor map of a stage input for TMA plane loads; false (registers only) where the
// field cannot take them: TMA off, rows not a multiple of 4 (a copy's row stride is a
// multiple of 16 bytes), a base address not 16-byte aligned, or no encoder.
bool encode_plane_map(CUtensorMap &tm, const float *f, const Grid &g)
{
    if (plane_loads.load() == 0) return false;
    if (g.rows % 4 != 0 || (reinterpret_cast<uintptr_t>(f) & 15u) != 0u) return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.rows, (cuuint64_t)g.cols, (cuuint64_t)g.pges};
    const cuuint64_t strides[2] = {(cuuint64_t)g.rows * 4u, (cuuint64_t)g.plane * 4u};
    const cuuint32_t box[3] = {(cuuint32_t)TMA_BOX_ROWS, (cuuint32_t)TMA_BOX_COLS, 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    return enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(f), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the RK stage is a template parameter of the tiled kernel (its combination and whether it
// reads the step-start field are then fixed at compile time); the ENORK2 kinds have two
template <int KIND, bool TMA>
void launch_stage_kind_as(int stage, dim3 gr, dim3 bl, cudaStream_t s, const TiledArgs &a, const CUtensorMap &tm)
{
    if constexpr (KIND == SK_VELOCITY) {
        k_stage_tiled<KIND, 0, TMA><<<gr, bl, 0, s>>>(a, tm);  // a single pass, not an RK stage
    } else if (stage == 0) {
        k_stage_tiled<KIND, 0, TMA><<<gr, bl, 0, s>>>(a, tm);
    } else if constexpr (KIND == SK_ENO2 || KIND == SK_ENO2R) {
        k_stage_tiled<KIND, 1, TMA><<<gr, bl, 0, s>>>(a, tm);
    } else {
        if (stage == 1)
            k_stage_tiled<KIND, 1, TMA><<<gr, bl, 0, s>>>(a, tm);
        else
            k_stage_tiled<KIND, 2, TMA><<<gr, bl, 0, s>>>(a, tm);
    }
}

template <int KIND> void launch_stage_kind(int stage, dim3 gr, dim3 bl, cudaStream_t s, const TiledArgs &a)
{
    CUtensorMap tm{};
    if (encode_plane_map(tm, a.phi_s, a.g))
        launch_stage_kind_as<KIND, true>(stage, gr, bl, s, a, tm);
    else
        launch_stage_kind_as<KIND, false>(stage, gr, bl, s, a, tm);
}

cudaError_t launch_tiled_stage(int kind, bool eno3, const TiledStage &st, const Grid &g, cudaStream_t s)
{
    TiledArgs a = tiled_args(g);
    a.phi_s = st.phi_s;
    a.phi_n = st.phi_n;
    a.out = st.out;
    a.flags = st.flags;
    a.d = st.d;
    a.v = st.v;
    a.speed = st.speed;
    a.dt = st.dt;
    unsigned *next = nullptr;
    if (static_band_kind(kind)) {
        a.queue = st.flagged.idx;
        a.counter = st.flagged.count;
    } else {
        a.queue = st.band.queue;
        a.counter = st.band.counter + (st.seq & 1);
        next = st.band.counter + ((st.seq + 1) & 1);
    }
    a.stage = st.stage;
    a.kz = tile_pages(g, kind);
    dim3 gr = tiled_grid(g, a.kz), bl(TY, TX);
    if (static_band_kind(kind)) {
        // the static band in the same launch: band blocks after the tile blocks
        a.sh = st.shadow;
        a.eno3 = eno3 ? 1 : 0;
        a.band_z = static_band_slabs(gr);
        gr.z += (unsigned)a.band_z;
        if (kind == SK_ENO2)
            launch_stage_kind<SK_ENO2>(a.stage, gr, bl, s, a);
        else if (kind == SK_ENO2R)
            launch_stage_kind<SK_ENO2R>(a.stage, gr, bl, s, a);
        else
            launch_stage_kind<SK_EXTEND>(a.stage, gr, bl, s, a);
        return cudaGetLastError();
    }
    if (kind == SK_REINIT)
        launch_stage_kind<SK_REINIT>(a.stage, gr, bl, s, a);
    else
        launch_stage_kind<SK_ADVECT>(a.stage, gr, bl, s, a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || kind == SK_ADVECT) return e;
    // the reinitialization's band is queued by the tiled kernel, so its kernel follows it
    if (eno3)
        k_band_stage<true><<<band_blocks(), 128, 0, s>>>(a, next);
    else
        k_band_stage<false><<<band_blocks(), 128, 0, s>>>(a, next);
    return cudaGetLastError();
}

// the extension velocity of the nodes without a distance flag on the tiles (the flagged
// nodes are k_velocity_list's)
cudaError_t launch_velocity_tiled(const float *phi, const uint8_t *flags, Ptr3<float> v, const Grid &g, float floor,
                                  cudaStream_t s)
{
    TiledArgs a = tiled_args(g);
    a.phi_s = phi;
    a.flags = flags;
    a.w = v;
    a.floor = floor;
    a.kz = tile_pages(g, SK_VELOCITY);
    launch_stage_kind<SK_VELOCITY>(0, tiled_grid(g, a.kz), dim3(TY, TX), s, a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// batched stages (k_stage_tiled_batch, k_band_stage_batch)
// ---------------------------------------------------------------------------------------
namespace {
// One block per work item: the hardware block scheduler hands items to SMs as blocks retire.
// (A persistent grid of the resident blocks walking the list grid-stride measured slower,
// 168 against 158 ms per step of the 64-vesicle batch: its static split left SMs idle at
// the end of each launch.)
template <int KIND> cudaError_t launch_batch_kind(int stage, const TiledBatch &B, int total, cudaStream_t s)
{
    const dim3 bl(TY, TX);
    auto go = [&](auto kernel) {
        kernel<<<total, bl, 0, s>>>(B);
        return cudaGetLastError();
    };
    if (stage == 0) return go(k_stage_tiled_batch<KIND, 0>);
    if constexpr (KIND == SK_ENO2 || KIND == SK_ENO2R) {
        return go(k_stage_tiled_batch<KIND, 1>);
    } else {
        if (stage == 1) return go(k_stage_tiled_batch<KIND, 1>);
        return go(k_stage_tiled_batch<KIND, 2>);
    }
}
}  // namespace

cudaError_t launch_tiled_batch(int kind, bool eno3, const TiledStage *st, const Grid *grids, int count, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    if (count > BATCH_MAX) return cudaErrorInvalidValue;
    // the tables are large (kernel parameters of ~16 and ~21 KB): one per host thread
    static thread_local TiledBatch B;
    static thread_local BandBatch BB;
    B.count = BB.count = count;
    int total = 0;
    for (int v = 0; v < count; ++v) {
        const Grid &g = grids[v];
        TiledArgs a = tiled_args(g);
        a.phi_s = st[v].phi_s;
        a.phi_n = st[v].phi_n;
        a.out = st[v].out;
        a.flags = st[v].flags;
        a.d = st[v].d;
        a.v = st[v].v;
        a.speed = st[v].speed;
        a.dt = st[v].dt;
        unsigned *next = nullptr;
        if (static_band_kind(kind)) {
            a.queue = st[v].flagged.idx;
            a.counter = st[v].flagged.count;
        } else {
            a.queue = st[v].band.queue;
            a.counter = st[v].band.counter + (st[v].seq & 1);
            next = st[v].band.counter + ((st[v].seq + 1) & 1);
        }
        a.stage = st[v].stage;
        a.kz = tile_pages(g, kind);
        a.sh = st[v].shadow;
        a.eno3 = eno3 ? 1 : 0;
        const dim3 gr = tiled_grid(g, a.kz);
        B.v[v] = a;
        B.nx[v] = (int)gr.x;
        B.ny[v] = (int)gr.y;
        B.start[v] = total;
        B.tiles[v] = (int)(gr.x * gr.y * gr.z);
        // static-band kinds: band blocks for a band of about 3% of the nodes, one node per
        // thread (a larger band is walked grid-stride)
        const long long nodes = (long long)g.rows * g.cols * g.pges;
        B.nb[v] = static_band_kind(kind) ? (int)std::max<long long>(1, (nodes * 3 / 100 + TY * TX - 1) / (TY * TX)) : 0;
        total += B.tiles[v] + B.nb[v];
        BB.v[v] = a;
        BB.next[v] = next;
    }
    B.start[count] = total;
    const int stage = st[0].stage;
    const int bgrid = band_blocks();
    cudaError_t e;
    if (static_band_kind(kind)) {
        if (kind == SK_ENO2) return launch_batch_kind<SK_ENO2>(stage, B, total, s);
        if (kind == SK_ENO2R) return launch_batch_kind<SK_ENO2R>(stage, B, total, s);
        return launch_batch_kind<SK_EXTEND>(stage, B, total, s);
    }
    e = kind == SK_REINIT ? launch_batch_kind<SK_REINIT>(stage, B, total, s) : launch_batch_kind<SK_ADVECT>(stage, B, total, s);
    if (e != cudaSuccess || kind == SK_ADVECT) return e;
    if (eno3)
        k_band_stage_batch<true><<<bgrid, 128, 0, s>>>(BB);
    else
        k_band_stage_batch<false><<<bgrid, 128, 0, s>>>(BB);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// set-up of the mixed form's extension band: FP64 crossing values and the shadows
// ---------------------------------------------------------------------------------------
namespace {
// crossing values at the listed nodes (boundary_interpolant.cu:78-141 /
// wenork3_extend.cu:296-365): the degree-5 / cubic interpolant of the promoted FP32
// values in FP64, product (Lagrange) form
template <bool CUBIC>
__global__ void __launch_bounds__(128) k_crossing_mixed(const float *__restrict__ cfield, Ptr6<const float> d,
                                                        Ptr6<double> cp, NodeList list, Grid g)
{
    const unsigned n = *list.count;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const long long c = list.idx[t];
        int i, j, k;
        node_of(g, c, i, j, k);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const float hf = (float)axis_h(g, ax);
            const float r1 = __ldg(d.p[2 * ax] + c), l1 = __ldg(d.p[2 * ax + 1] + c);
            double cf = 0.0, cb = 0.0;
            if (r1 < hf || l1 < hf) {
                const AxisLine L = axis_line(g, i, j, k, ax);
                double p[7];
#pragma unroll
                for (int s = -3; s <= 3; ++s)
                    p[s + 3] = (double)__ldg(cfield + L.base + (long long)clampi(L.c + s, L.n) * L.stride);
                const double h = (double)hf, rf = (double)r1, rb = (double)l1;
                if (CUBIC) {
                    if (r1 < hf) cf = lagrange_equispaced<4, double>(p + 2, 1.0 + rf / h);
                    if (l1 < hf) cb = lagrange_equispaced<4, double>(p + 1, 2.0 - rb / h);
                } else {
                    if (r1 < hf) cf = lagrange_equispaced<6, double>(p + 1, 2.0 + rf / h);
                    if (l1 < hf) cb = lagrange_equispaced<6, double>(p, 3.0 - rb / h);
                }
            }
            cp.p[2 * ax][c] = cf;
            cp.p[2 * ax + 1][c] = cb;
        }
    }
}

// ENORK2 crossing values (enork2_extend.cu:144-211) in FP64 on the promoted FP32 values
__global__ void __launch_bounds__(128) k_enork2_crossing_mixed(const float *__restrict__ cfield, Ptr6<const float> d,
                                                               Ptr6<double> cp, NodeList list, Grid g)
{
    const unsigned n = *list.count;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const long long c = list.idx[t];
        int i, j, k;
        node_of(g, c, i, j, k);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const AxisLine L = axis_line(g, i, j, k, ax);
            double p[7], cf, cb;
#pragma unroll
            for (int s = -3; s <= 3; ++s)
                p[s + 3] = (double)__ldg(cfield + L.base + (long long)clampi(L.c + s, L.n) * L.stride);
            const float hf = (float)axis_h(g, ax);
            const float r1 = __ldg(d.p[2 * ax] + c), l1 = __ldg(d.p[2 * ax + 1] + c);
            // the tests r1 != h, l1 != h of the FP32 distances hold unchanged once promoted
            eno2_crossing<double>(p, (double)r1, (double)l1, (double)hf, cf, cb);
            cp.p[2 * ax][c] = cf;
            cp.p[2 * ax + 1][c] = cb;
        }
    }
}

__global__ void __launch_bounds__(128) k_shadow_init(const float *__restrict__ c, double *__restrict__ shadow,
                                                     NodeList list)
{
    const unsigned n = *list.count;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const unsigned q = list.idx[t];
        shadow[q] = (double)__ldg(c + q);
    }
}
}  // namespace

cudaError_t launch_crossing_mixed(const float *c, Ptr6<const float> dist, Ptr6<double> cp, NodeList list,
                                  const Grid &g, bool cubic, cudaStream_t s)
{
    if (cubic)
        k_crossing_mixed<true><<<list_blocks(), 128, 0, s>>>(c, dist, cp, list, g);
    else
        k_crossing_mixed<false><<<list_blocks(), 128, 0, s>>>(c, dist, cp, list, g);
    return cudaGetLastError();
}

cudaError_t launch_enork2_crossing_mixed(const float *c, Ptr6<const float> dist, Ptr6<double> cp, NodeList list,
                                         const Grid &g, cudaStream_t s)
{
    k_enork2_crossing_mixed<<<list_blocks(), 128, 0, s>>>(c, dist, cp, list, g);
    return cudaGetLastError();
}

cudaError_t launch_shadow_init(const float *c, double *shadow, NodeList list, cudaStream_t s)
{
    k_shadow_init<<<list_blocks(), 128, 0, s>>>(c, shadow, list);
    return cudaGetLastError();
}

}  // namespace vsl
