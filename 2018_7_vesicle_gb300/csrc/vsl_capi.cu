// vsl_capi.cu -- method-level entry points of the C ABI (include/vsl_gb300.h): argument
// checks, workspace carving and the launch sequences of the TVD-RK3 loops.  Everything
// is enqueued on the caller's stream; nothing here allocates or synchronises.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>

#include "vsl_internal.h"

namespace vsl {
namespace {

// ---------------------------------------------------------------------------------------
// workspace: a bump allocator over the caller's buffer (256-byte aligned pieces); with a
// null base it only measures
// ---------------------------------------------------------------------------------------
struct Bump {
    char *base;
    size_t used = 0;
    explicit Bump(void *b) : base(static_cast<char *>(b)) {}
    template <typename U> U *take(long long n)
    {
        used = (used + 255) & ~size_t(255);
        U *p = base ? reinterpret_cast<U *>(base + used) : nullptr;
        used += sizeof(U) * (size_t)n;
        return p;
    }
};

// band queue of the tiled FP32 kernels (allocated for FP32 only) and its stage count
struct Band {
    BandQueue q{nullptr, nullptr};
    int seq = 0;
};
template <typename T> Band carve_band(Bump &w, const Grid &g)
{
    Band b;
    if (std::is_same<T, float>::value) {
        b.q.queue = w.take<unsigned>(g.num);
        b.q.counter = w.take<unsigned>(2);
    }
    return b;
}

EdgeLists carve_edges(Bump &w, const Grid &g)
{
    EdgeLists e;
    for (int q = 0; q < 3; ++q) e.idx[q] = w.take<unsigned>(g.num);
    e.count = w.take<unsigned>(4);
    return e;
}
NodeList carve_list(Bump &w, const Grid &g)
{
    NodeList l;
    l.idx = w.take<unsigned>(g.num);
    l.count = w.take<unsigned>(1);
    return l;
}

template <typename T> struct ReinitWork {
    T *b, *c;
    uint8_t *flags;
    Ptr6<T> dist;     // ENO3 only
    EdgeLists edges;  // ENO3 only (its setDistance)
    Band band;
};
template <typename T> ReinitWork<T> carve_reinit(Bump &w, const Grid &g, bool own_dist)
{
    ReinitWork<T> r{};
    r.b = w.take<T>(g.num);
    r.c = w.take<T>(g.num);
    r.flags = w.take<uint8_t>(g.num);
    for (int q = 0; q < 6; ++q) r.dist.p[q] = own_dist ? w.take<T>(g.num) : nullptr;
    r.edges = own_dist ? carve_edges(w, g) : EdgeLists{};
    r.band = carve_band<T>(w, g);
    return r;
}

template <typename T> struct ExtendWork {
    Ptr3<T> v;
    Ptr6<T> cp;         // FP64 form: crossing values
    Ptr6<double> cp64;  // FP32 form: FP64 crossing values and the band's shadow fields
    double *sh[3];
    T *b, *c;
    uint8_t *flags;
    NodeList flagged;  // nodes with a distance flag: crossing values and the band
    Ptr6<T> dist;      // ENO3 only
    EdgeLists edges;   // ENO3 only (its setDistance)
    Band band;
};
template <typename T> ExtendWork<T> carve_extend(Bump &w, const Grid &g, bool own_dist)
{
    ExtendWork<T> e{};
    for (int q = 0; q < 3; ++q) e.v.p[q] = w.take<T>(g.num);
    if (std::is_same<T, float>::value) {
        for (int q = 0; q < 6; ++q) e.cp64.p[q] = w.take<double>(g.num);
        for (int q = 0; q < 3; ++q) e.sh[q] = w.take<double>(g.num);
    } else {
        for (int q = 0; q < 6; ++q) e.cp.p[q] = w.take<T>(g.num);
    }
    e.b = w.take<T>(g.num);
    e.c = w.take<T>(g.num);
    e.flags = w.take<uint8_t>(g.num);
    e.flagged = carve_list(w, g);
    for (int q = 0; q < 6; ++q) e.dist.p[q] = own_dist ? w.take<T>(g.num) : nullptr;
    e.edges = own_dist ? carve_edges(w, g) : EdgeLists{};
    e.band = carve_band<T>(w, g);
    return e;
}

// the residual-driven reinitialization: the reinitialization workspace and the residual's
// two reduction words
template <typename T> struct TolWork {
    ReinitWork<T> re;
    unsigned long long *max_bits;
    unsigned *ticket;
};
template <typename T> TolWork<T> carve_tol(Bump &w, const Grid &g)
{
    TolWork<T> t;
    t.re = carve_reinit<T>(w, g, false);
    t.max_bits = w.take<unsigned long long>(2);  // the ticket shares the second word
    t.ticket = t.max_bits ? reinterpret_cast<unsigned *>(t.max_bits + 1) : nullptr;
    return t;
}

// zero the band counters before the first tiled stage of an operation
int band_reset(Band &b, cudaStream_t s)
{
    b.seq = 0;
    if (b.q.counter == nullptr) return VSL_OK;
    return cudaMemsetAsync(b.q.counter, 0, 2 * sizeof(unsigned), s) == cudaSuccess ? VSL_OK : VSL_ERR_CUDA;
}

template <typename T> struct RedistWork {
    ExtendWork<T> ext;  // F's distances in ext.dist
    ReinitWork<T> re;   // A's distances in re.dist
};
template <typename T> RedistWork<T> carve_redist(Bump &w, const Grid &g)
{
    RedistWork<T> r;
    r.ext = carve_extend<T>(w, g, true);
    r.re = carve_reinit<T>(w, g, true);
    return r;
}

struct ReduceWork {
    double *partials;
    double *scalars;  // dt, vmax
};
ReduceWork carve_reduce(Bump &w, const Grid &g, int ncomp)
{
    ReduceWork r;
    r.partials = w.take<double>((long long)ncomp * toolbox_partial_blocks(g));
    r.scalars = w.take<double>(4);
    return r;
}

// the per-node values pass 2 of the auxiliary toolbox reads, where the caller does not
// ask for them as outputs (sized for all of them)
template <typename T> AuxKeep<T> carve_aux(Bump &w, const Grid &g)
{
    AuxKeep<T> k;
    k.cx = w.take<T>(g.num);
    k.cy = w.take<T>(g.num);
    k.cz = w.take<T>(g.num);
    k.ncr = w.take<T>(g.num);
    k.agm = w.take<T>(g.num);
    k.adelta = w.take<T>(g.num);
    k.aheav = w.take<T>(g.num);
    k.fheav = w.take<T>(g.num);
    return k;
}

template <typename T> struct StepWork {
    T *vn;
    Ptr3<T> nrm;
    ExtendWork<T> ext;
    ReduceWork red;
    EdgeLists edges;
};
template <typename T> StepWork<T> carve_step(Bump &w, const Grid &g)
{
    StepWork<T> s;
    s.vn = w.take<T>(g.num);
    for (int q = 0; q < 3; ++q) s.nrm.p[q] = w.take<T>(g.num);
    s.ext = carve_extend<T>(w, g, false);
    s.red = carve_reduce(w, g, 2);
    s.edges = carve_edges(w, g);
    return s;
}

// adjoint sweeps: recomputed stage fields b, c (inside `re`), the 21 Jacobian slots,
// the running adjoint x, the RK3 base accumulator and (reinitialization) the six
// distance adjoints
template <typename T> struct AdjWork {
    ReinitWork<T> re;
    T *W, *x, *acc;
    Ptr6<T> mu;
    NodeList band;  // reinitialization: nodes next to a sign change
};
template <typename T> AdjWork<T> carve_adj(Bump &w, const Grid &g, bool reinit)
{
    AdjWork<T> a{};
    a.re = carve_reinit<T>(w, g, reinit);
    a.W = w.take<T>((long long)ADJ_SLOTS * g.num);
    a.x = w.take<T>(g.num);
    a.acc = w.take<T>(g.num);
    for (int q = 0; q < 6; ++q) a.mu.p[q] = reinit ? w.take<T>(g.num) : nullptr;
    a.band = reinit ? carve_list(w, g) : NodeList{nullptr, nullptr};
    return a;
}

// spectral smoothing: the complex spectrum and cuFFT's work area
template <typename T> struct SpecWork {
    void *spec = nullptr;
    void *work = nullptr;
    size_t work_bytes = 0;
};
template <typename T> SpecWork<T> carve_spec(Bump &w, const Grid &g)
{
    SpecWork<T> sp;
    sp.spec = w.take<T>(2 * g.num);
    sp.work_bytes = spectral_work_bytes<T>(g);
    sp.work = w.take<char>((long long)sp.work_bytes);
    return sp;
}

// relaxation step: toolbox outputs (H extended in place), bending and normal speeds, the
// extensions, reductions, setDistance's edge lists, the reinitialization and smoothing
template <typename T> struct RelaxWork {
    T *H, *K, *G, *D, *nsb, *vn;
    ExtendWork<T> ext;
    ReduceWork red;
    EdgeLists edges;
    ReinitWork<T> re;
    SpecWork<T> spec;
};
template <typename T> RelaxWork<T> carve_relax(Bump &w, const Grid &g)
{
    RelaxWork<T> r;
    r.H = w.take<T>(g.num);
    r.K = w.take<T>(g.num);
    r.G = w.take<T>(g.num);
    r.D = w.take<T>(g.num);
    r.nsb = w.take<T>(g.num);
    r.vn = w.take<T>(g.num);
    r.ext = carve_extend<T>(w, g, true);
    r.red = carve_reduce(w, g, 4);
    r.edges = carve_edges(w, g);
    r.re = carve_reinit<T>(w, g, false);
    r.spec = carve_spec<T>(w, g);
    return r;
}

size_t measure(int op, const Grid &g, int elem)
{
    Bump w(nullptr);
    auto run = [&](auto tag) {
        using T = decltype(tag);
        switch (op) {
        case VSL_OP_REINIT_WENO5: carve_reinit<T>(w, g, false); break;
        case VSL_OP_REINIT_ENO3: carve_reinit<T>(w, g, true); break;
        case VSL_OP_EXTEND_WENO5: carve_extend<T>(w, g, false); break;
        case VSL_OP_EXTEND_ENO3: carve_extend<T>(w, g, true); break;
        case VSL_OP_SURFACE_REDISTANCE:
        case VSL_OP_SURFACE_REDISTANCE_ENO3: carve_redist<T>(w, g); break;
        case VSL_OP_AREA_VOLUME: carve_reduce(w, g, 2); break;
        case VSL_OP_ADVECTION: carve_reinit<T>(w, g, false); break;
        case VSL_OP_VESICLE_STEP: carve_step<T>(w, g); break;
        case VSL_OP_SET_DISTANCE: carve_edges(w, g); break;
        case VSL_OP_ADVECTION_ADJOINT: carve_adj<T>(w, g, false); break;
        case VSL_OP_REINIT_ADJOINT: carve_adj<T>(w, g, true); break;
        case VSL_OP_REINIT_ENORK2: carve_reinit<T>(w, g, true); break;
        case VSL_OP_EXTEND_ENORK2: carve_extend<T>(w, g, true); break;
        case VSL_OP_SURFACE_REDISTANCE_ENORK2: carve_redist<T>(w, g); break;
        case VSL_OP_SMOOTH: {
            SpecWork<T> sp = carve_spec<T>(w, g);
            if (sp.work_bytes == 0 && g.num > 0) w.take<char>(1);  // plan creation failed: keep a size
            break;
        }
        case VSL_OP_RELAX_STEP: carve_relax<T>(w, g); break;
        case VSL_OP_AUX_TOOLBOX: carve_aux<T>(w, g); break;
        case VSL_OP_MASKED_INTEGRAL: carve_reduce(w, g, 1); break;
        case VSL_OP_REINIT_TOL: carve_tol<T>(w, g); break;
        default: return false;
        }
        return true;
    };
    bool ok = elem == 8 ? run(double{}) : (elem == 4 ? run(float{}) : false);
    return ok ? ((w.used + 255) & ~size_t(255)) : 0;
}

// ---------------------------------------------------------------------------------------
// checks
// ---------------------------------------------------------------------------------------
template <typename... P> bool any_null(P... p) { return ((p == nullptr) || ...); }

int check_ws(int op, const Grid &g, int elem, void *ws, size_t bytes)
{
    if (ws == nullptr) return VSL_ERR_WORKSPACE;
    if (reinterpret_cast<uintptr_t>(ws) % 256 != 0) return VSL_ERR_WORKSPACE;
    if (bytes < measure(op, g, elem)) return VSL_ERR_WORKSPACE;
    return VSL_OK;
}

#define VSL_TRY(expr)                                                                                              \
    do {                                                                                                           \
        cudaError_t e_ = (expr);                                                                                   \
        if (e_ != cudaSuccess) return VSL_ERR_CUDA;                                                                \
    } while (0)
#define VSL_TRY_CUDA(expr)                                                                                         \
    do {                                                                                                           \
        cudaError_t e_ = (expr);                                                                                   \
        if (e_ != cudaSuccess) return e_;                                                                          \
    } while (0)

template <typename T> constexpr bool fast_form() { return std::is_same<T, float>::value; }

template <typename T> Ptr6<const T> cview(const Ptr6<T> &p)
{
    Ptr6<const T> r;
    for (int q = 0; q < 6; ++q) r.p[q] = p.p[q];
    return r;
}
template <typename T> Ptr3<const T> cview3(const Ptr3<T> &p)
{
    Ptr3<const T> r;
    for (int q = 0; q < 3; ++q) r.p[q] = p.p[q];
    return r;
}

// ---------------------------------------------------------------------------------------
// loops
// ---------------------------------------------------------------------------------------

// one stage through the tiled FP32 kernels (stage input s_in, RK3 base n_in, output out)
inline cudaError_t tiled(int kind, bool eno3, Band &band, const float *s_in, const float *n_in, float *out,
                         const uint8_t *flags, Ptr6<const float> d, BandShadow sh, Ptr3<const float> v,
                         const float *speed, const double *dt, int stage, const Grid &g, cudaStream_t s,
                         NodeList flagged = NodeList{nullptr, nullptr})
{
    TiledStage st{s_in, n_in, out, flags, d, sh, v, speed, dt, band.q, flagged, stage, band.seq++};
    return launch_tiled_stage(kind, eno3, st, g, s);
}

// `iters` TVD-RK3 reinitialization pseudo-steps of F in place (flags already classified)
template <typename T>
int reinit_loop(T *F, int iters, Ptr6<const T> d, ReinitWork<T> &w, const Grid &g, bool eno3, cudaStream_t s)
{
    const bool fast = fast_form<T>();
    if constexpr (std::is_same<T, float>::value) {
        if (int st = band_reset(w.band, s)) return st;
        const BandShadow none{};
        const Ptr3<const float> none3{};
        for (int it = 0; it < iters; ++it) {
            VSL_TRY(tiled(0, eno3, w.band, F, F, w.b, w.flags, d, none, none3, nullptr, nullptr, 0, g, s));
            VSL_TRY(tiled(0, eno3, w.band, w.b, F, w.c, w.flags, d, none, none3, nullptr, nullptr, 1, g, s));
            VSL_TRY(tiled(0, eno3, w.band, w.c, F, F, w.flags, d, none, none3, nullptr, nullptr, 2, g, s));
        }
        return VSL_OK;
    } else {
        for (int it = 0; it < iters; ++it) {
            VSL_TRY(launch_reinit_stage<T>(F, F, w.b, w.flags, d, g, 0, eno3, fast, s));
            VSL_TRY(launch_reinit_stage<T>(w.b, F, w.c, w.flags, d, g, 1, eno3, fast, s));
            VSL_TRY(launch_reinit_stage<T>(w.c, F, F, w.flags, d, g, 2, eno3, fast, s));
        }
        return VSL_OK;
    }
}

// one TVD-RK3 reinitialization pseudo-step of F in place, kernel launches only (the FP32
// band counters must be zero, as band_reset leaves them; the third stage leaves counter 0
// set and counter 1 zero)
template <typename T>
int reinit_pseudo_step(T *F, Ptr6<const T> d, ReinitWork<T> &w, const Grid &g, cudaStream_t s)
{
    if constexpr (std::is_same<T, float>::value) {
        const BandShadow none{};
        const Ptr3<const float> none3{};
        w.band.seq = 0;
        VSL_TRY(tiled(0, false, w.band, F, F, w.b, w.flags, d, none, none3, nullptr, nullptr, 0, g, s));
        VSL_TRY(tiled(0, false, w.band, w.b, F, w.c, w.flags, d, none, none3, nullptr, nullptr, 1, g, s));
        VSL_TRY(tiled(0, false, w.band, w.c, F, F, w.flags, d, none, none3, nullptr, nullptr, 2, g, s));
    } else {
        VSL_TRY(launch_reinit_stage<T>(F, F, w.b, w.flags, d, g, 0, false, false, s));
        VSL_TRY(launch_reinit_stage<T>(w.b, F, w.c, w.flags, d, g, 1, false, false, s));
        VSL_TRY(launch_reinit_stage<T>(w.c, F, F, w.flags, d, g, 2, false, false, s));
    }
    return VSL_OK;
}

// velocity and node classes of an extension off the zero set of F (distances d)
template <typename T>
int extend_setup(const T *F, Ptr6<const T> d, const ExtendWork<T> &w, const Grid &g, bool eno3, double floor,
                 cudaStream_t s)
{
    VSL_TRY(launch_classify<T>(F, d, w.flags, w.flagged, g, s));
    VSL_TRY(launch_extension_velocity<T>(F, w.flags, d, w.v, g, eno3, floor, w.flagged, s));
    return VSL_OK;
}

// crossing values of C, then `iters` TVD-RK3 extension pseudo-steps of C in place
template <typename T>
int extend_loop(T *C, int iters, Ptr6<const T> d, ExtendWork<T> &w, const Grid &g, bool eno3, cudaStream_t s)
{
    const bool fast = fast_form<T>();
    Ptr3<const T> v = cview3(w.v);
    if constexpr (std::is_same<T, float>::value) {
        // FP64 crossing values and the band's FP64 shadow of C (BandShadow)
        VSL_TRY(launch_crossing_mixed(C, d, w.cp64, w.flagged, g, eno3, s));
        VSL_TRY(launch_shadow_init(C, w.sh[0], w.flagged, s));
        const Ptr6<const double> cp = cview(w.cp64);
        if (int st = band_reset(w.band, s)) return st;
        for (int it = 0; it < iters; ++it) {
            VSL_TRY(tiled(1, eno3, w.band, C, C, w.b, w.flags, d, BandShadow{w.sh[0], w.sh[0], w.sh[1], cp}, v,
                          nullptr, nullptr, 0, g, s, w.flagged));
            VSL_TRY(tiled(1, eno3, w.band, w.b, C, w.c, w.flags, d, BandShadow{w.sh[1], w.sh[0], w.sh[2], cp}, v,
                          nullptr, nullptr, 1, g, s, w.flagged));
            VSL_TRY(tiled(1, eno3, w.band, w.c, C, C, w.flags, d, BandShadow{w.sh[2], w.sh[0], w.sh[0], cp}, v,
                          nullptr, nullptr, 2, g, s, w.flagged));
        }
        return VSL_OK;
    } else {
        VSL_TRY(launch_crossing<T>(C, d, w.cp, w.flagged, g, eno3, s));
        Ptr6<const T> cp = cview(w.cp);
        for (int it = 0; it < iters; ++it) {
            VSL_TRY(launch_extend_stage<T>(C, C, w.b, w.flags, d, cp, v, g, 0, eno3, fast, s));
            VSL_TRY(launch_extend_stage<T>(w.b, C, w.c, w.flags, d, cp, v, g, 1, eno3, fast, s));
            VSL_TRY(launch_extend_stage<T>(w.c, C, C, w.flags, d, cp, v, g, 2, eno3, fast, s));
        }
        return VSL_OK;
    }
}

template <typename T>
int advect_loop(T *F, Ptr3<const T> v, const T *speed, const double *dt, int steps, ReinitWork<T> &w, const Grid &g,
                cudaStream_t s)
{
    const bool fast = fast_form<T>();
    if constexpr (std::is_same<T, float>::value) {
        const Ptr6<const float> none6{};
        for (int it = 0; it < steps; ++it) {
            VSL_TRY(tiled(2, false, w.band, F, F, w.b, nullptr, none6, BandShadow{}, v, speed, dt, 0, g, s));
            VSL_TRY(tiled(2, false, w.band, w.b, F, w.c, nullptr, none6, BandShadow{}, v, speed, dt, 1, g, s));
            VSL_TRY(tiled(2, false, w.band, w.c, F, F, nullptr, none6, BandShadow{}, v, speed, dt, 2, g, s));
        }
        return VSL_OK;
    } else {
        for (int it = 0; it < steps; ++it) {
            VSL_TRY(launch_advect_stage<T>(F, F, w.b, v, speed, dt, g, 0, fast, s));
            VSL_TRY(launch_advect_stage<T>(w.b, F, w.c, v, speed, dt, g, 1, fast, s));
            VSL_TRY(launch_advect_stage<T>(w.c, F, F, v, speed, dt, g, 2, fast, s));
        }
        return VSL_OK;
    }
}

template <typename T> Ptr6<const T> six(const T *a, const T *b, const T *c, const T *d, const T *e, const T *f)
{
    return Ptr6<const T>{{a, b, c, d, e, f}};
}

// ---------------------------------------------------------------------------------------
// operations (templated on the field type)
// ---------------------------------------------------------------------------------------

template <typename T>
int op_set_distance(const T *F, T *xpr, T *xpl, T *ypf, T *ypb, T *zpu, T *zpd, int rows, int cols, int pges,
                    double dx, double dy, double dz, void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F, xpr, xpl, ypf, ypb, zpu, zpd)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_SET_DISTANCE, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    EdgeLists e = carve_edges(b, g);
    VSL_TRY(launch_set_distance<T>(F, Ptr6<T>{{xpr, xpl, ypf, ypb, zpu, zpd}}, g, true, e, s));
    return VSL_OK;
}

template <typename T>
int op_reinit_weno5(T *F, int iteration, const T *xpr, const T *xpl, const T *ypf, const T *ypb, const T *zpu,
                    const T *zpd, int rows, int cols, int pges, double dx, double dy, double dz, void *ws,
                    size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F, xpr, xpl, ypf, ypb, zpu, zpd)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (iteration < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_REINIT_WENO5, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    ReinitWork<T> w = carve_reinit<T>(b, g, false);
    Ptr6<const T> d = six(xpr, xpl, ypf, ypb, zpu, zpd);
    VSL_TRY(launch_classify<T>(F, d, w.flags, NodeList{nullptr, nullptr}, g, s));
    return reinit_loop<T>(F, iteration, d, w, g, false, s);
}

template <typename T>
int op_reinit_eno3(T *F, int iteration, int rows, int cols, int pges, double dx, double dy, double dz, void *ws,
                   size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (iteration < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_REINIT_ENO3, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    ReinitWork<T> w = carve_reinit<T>(b, g, true);
    VSL_TRY(launch_set_distance<T>(F, w.dist, g, false, w.edges, s));
    Ptr6<const T> d = cview(w.dist);
    VSL_TRY(launch_classify<T>(F, d, w.flags, NodeList{nullptr, nullptr}, g, s));
    return reinit_loop<T>(F, iteration, d, w, g, true, s);
}

template <typename T>
int op_extend_weno5(T *C, int iteration, const T *F, const T *xpr, const T *xpl, const T *ypf, const T *ypb,
                    const T *zpu, const T *zpd, int rows, int cols, int pges, double dx, double dy, double dz,
                    void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(C, F, xpr, xpl, ypf, ypb, zpu, zpd)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (iteration < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_EXTEND_WENO5, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    ExtendWork<T> w = carve_extend<T>(b, g, false);
    Ptr6<const T> d = six(xpr, xpl, ypf, ypb, zpu, zpd);
    if (int st = extend_setup<T>(F, d, w, g, false, 1e-6, s)) return st;
    return extend_loop<T>(C, iteration, d, w, g, false, s);
}

template <typename T>
int op_extend_eno3(T *C, int iteration, const T *F, int rows, int cols, int pges, double dx, double dy, double dz,
                   void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(C, F)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (iteration < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_EXTEND_ENO3, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    ExtendWork<T> w = carve_extend<T>(b, g, true);
    VSL_TRY(launch_set_distance<T>(F, w.dist, g, false, w.edges, s));
    Ptr6<const T> d = cview(w.dist);
    if (int st = extend_setup<T>(F, d, w, g, true, 1e-6, s)) return st;
    return extend_loop<T>(C, iteration, d, w, g, true, s);
}

// WENO5RK3ClosetPointSurfaceRedistance.m:4-157 (eno3 = false) and its WENORK3 form,
// WENORK3ClosetPointSurfaceRedistance.m:4-152 (eno3 = true): the same composition with
// the cubic distances, the WENORK3 upwind normals, crossing values and extension step and
// the ENO3 interface scheme of the reinitialization
template <typename T>
int op_redistance(T *A, int iter1, int iter2, const T *F, int rows, int cols, int pges, double dx, double dy,
                  double dz, bool eno3, void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(A, F)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (iter1 < 0 || iter2 < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    const int op = eno3 ? VSL_OP_SURFACE_REDISTANCE_ENO3 : VSL_OP_SURFACE_REDISTANCE;
    if (int st = check_ws(op, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    RedistWork<T> w = carve_redist<T>(b, g);
    // reinitialization part: distances of A, mask A < 0 (ClosetPointSurfaceRedistance.m:15-25)
    VSL_TRY(launch_set_distance<T>(A, w.re.dist, g, !eno3, w.re.edges, s));
    Ptr6<const T> dA = cview(w.re.dist);
    VSL_TRY(launch_classify<T>(A, dA, w.re.flags, NodeList{nullptr, nullptr}, g, s));
    // extension part: distances and upwind normals of F, floor 1e-14 (:37-74)
    VSL_TRY(launch_set_distance<T>(F, w.ext.dist, g, !eno3, w.ext.edges, s));
    Ptr6<const T> dF = cview(w.ext.dist);
    if (int st = extend_setup<T>(F, dF, w.ext, g, eno3, 1e-14, s)) return st;
    const bool fast = fast_form<T>();
    if (int st = band_reset(w.re.band, s)) return st;
    // one reinitialization stage of A's pseudo-time loop (tiled kernels for FP32)
    auto re_stage = [&](const T *in, T *out, int stage) -> cudaError_t {
        if constexpr (std::is_same<T, float>::value)
            return tiled(0, eno3, w.re.band, in, A, out, w.re.flags, dA, BandShadow{}, Ptr3<const float>{},
                         nullptr, nullptr, stage, g, s);
        else
            return launch_reinit_stage<T>(in, A, out, w.re.flags, dA, g, stage, eno3, fast, s);
    };
    // the reinit stages need their own temporaries: the extension uses w.ext.b/c
    T *t1 = w.re.b, *t2 = w.re.c;
    for (int it = 0; it < iter1; ++it) {
        if (int st = extend_loop<T>(A, iter2, dF, w.ext, g, eno3, s)) return st;
        VSL_TRY(re_stage(A, t1, 0));
        if (int st = extend_loop<T>(t1, iter2, dF, w.ext, g, eno3, s)) return st;
        VSL_TRY(re_stage(t1, t2, 1));
        if (int st = extend_loop<T>(t2, iter2, dF, w.ext, g, eno3, s)) return st;
        VSL_TRY(re_stage(t2, A, 2));
    }
    return extend_loop<T>(A, iter2, dF, w.ext, g, eno3, s);
}

template <typename T>
int op_area_volume(const T *F, double *av, int rows, int cols, int pges, double dx, double dy, double dz, void *ws,
                   size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F, av)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_AREA_VOLUME, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    ReduceWork r = carve_reduce(b, g, 2);
    const double ds = (dx + dy + dz) / 3;
    ToolboxOut<T> none{};
    int nb = 0;
    VSL_TRY(launch_toolbox<T>(F, none, g, ds, r.partials, &nb, s));
    VSL_TRY(launch_sum_partials(r.partials, nb, 2, std::pow(ds, 3), av, s));
    return VSL_OK;
}

// GPUAsetCalculusToolBox.m:2-63 for the auxiliary level set A on F: out holds the 27 fields
// of auxi_set_calculus_toolbox, then AFDiracDelta and ADiracDeltaDn; null entries are not
// written.
template <typename T>
int op_aux_toolbox(const T *A, const T *F, T *const *out, int rows, int cols, int pges, double dx, double dy,
                   double dz, void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(A, F, out)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_AUX_TOOLBOX, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    AuxKeep<T> keep = carve_aux<T>(b, g);
    AuxOut<T> o;
    for (int q = 0; q < AUX_OUT_FIELDS; ++q) o.f[q] = out[q];
    // pass 2 reads the caller's arrays where the caller asked for those fields
    if (o.f[4]) keep.cx = o.f[4];
    if (o.f[5]) keep.cy = o.f[5];
    if (o.f[6]) keep.cz = o.f[6];
    if (o.f[7]) keep.ncr = o.f[7];
    if (o.f[3]) keep.agm = o.f[3];
    if (o.f[26]) keep.adelta = o.f[26];
    if (o.f[25]) keep.aheav = o.f[25];
    VSL_TRY(launch_aux_toolbox<T>(A, F, o, keep, g, (dx + dy + dz) / 3, s));
    return VSL_OK;
}

// sum over |F| < 2Ds (and |A| < 2Ds where A is given) of ((f0 f1) f2) (1 - one_minus) Ds^3,
// the factors that are given, in FP64 (SDF3.m:82-85, 212-227)
template <typename T>
int op_masked_integral(const T *F, const T *A, const T *f0, const T *f1, const T *f2, const T *one_minus,
                       double *result, int rows, int cols, int pges, double dx, double dy, double dz, void *ws,
                       size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F, result)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_MASKED_INTEGRAL, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    ReduceWork r = carve_reduce(b, g, 1);
    const double ds = (dx + dy + dz) / 3;
    int nb = 0;
    VSL_TRY(launch_masked_sum<T>(F, A, f0, f1, f2, one_minus, g, ds, r.partials, &nb, s));
    VSL_TRY(launch_sum_partials(r.partials, nb, 1, std::pow(ds, 3), result, s));
    return VSL_OK;
}

template <typename T>
int op_advection(T *F, const T *vx, const T *vy, const T *vz, const double *dt, int steps, int rows, int cols,
                 int pges, double dx, double dy, double dz, void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F, vx, vy, vz, dt)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (steps < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_ADVECTION, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    ReinitWork<T> w = carve_reinit<T>(b, g, false);
    return advect_loop<T>(F, Ptr3<const T>{{vx, vy, vz}}, nullptr, dt, steps, w, g, s);
}

template <typename T>
int op_vesicle_step(T *F, T *xpr, T *xpl, T *ypf, T *ypb, T *zpu, T *zpd, int ext_iters, int reinit_iters,
                    double cfl, double *info, int rows, int cols, int pges, double dx, double dy, double dz, void *ws,
                    size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F, xpr, xpl, ypf, ypb, zpu, zpd, info)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (ext_iters < 0 || reinit_iters < 0 || !(cfl > 0)) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_VESICLE_STEP, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    StepWork<T> w = carve_step<T>(b, g);
    const double ds = (dx + dy + dz) / 3;
    Ptr6<const T> d = six<T>(xpr, xpl, ypf, ypb, zpu, zpd);
    // calculus toolbox: mean curvature (the normal speed), normals, area and volume
    ToolboxOut<T> tb{};
    tb.f[4] = w.nrm.p[0];
    tb.f[5] = w.nrm.p[1];
    tb.f[6] = w.nrm.p[2];
    tb.f[14] = w.vn;
    int nb = 0;
    VSL_TRY(launch_toolbox<T>(F, tb, g, ds, w.red.partials, &nb, s));
    VSL_TRY(launch_sum_partials(w.red.partials, nb, 2, std::pow(ds, 3), info, s));
    // extend the normal speed off the interface (cached distances of F)
    if (int st = extend_setup<T>(F, d, w.ext, g, false, 1e-6, s)) return st;
    if (int st = extend_loop<T>(w.vn, ext_iters, d, w.ext, g, false, s)) return st;
    // dt = cfl * Ds / max |Vn| over |F| < 2 Ds
    VSL_TRY(launch_band_maxabs<T>(w.vn, F, 2 * ds, g, w.red.partials, &nb, s));
    VSL_TRY(launch_time_step(w.red.partials, nb, cfl * ds, info + 2, info + 3, s));
    // one WENO5 TVD-RK3 advection step along Vn * N
    ReinitWork<T> tmp{};
    tmp.b = w.ext.b;
    tmp.c = w.ext.c;
    tmp.band = w.ext.band;
    if (int st = advect_loop<T>(F, cview3(w.nrm), w.vn, info + 2, 1, tmp, g, s)) return st;
    // setDistance, then reinitialization
    VSL_TRY(launch_set_distance<T>(F, Ptr6<T>{{xpr, xpl, ypf, ypb, zpu, zpd}}, g, true, w.edges, s));
    ReinitWork<T> rw{};
    rw.b = w.ext.b;
    rw.c = w.ext.c;
    rw.flags = w.ext.flags;
    rw.band = w.ext.band;
    VSL_TRY(launch_classify<T>(F, d, rw.flags, NodeList{nullptr, nullptr}, g, s));
    return reinit_loop<T>(F, reinit_iters, d, rw, g, false, s);
}

// ---------------------------------------------------------------------------------------
// residual-driven reinitialization (no counterpart in the reference, whose loop runs a
// fixed count, WENO5RK3Reinitialization.m:15).  One CUDA graph: a prelude (classification,
// the residual of the input) and a conditional WHILE node whose body is one pseudo-step
// followed by the residual, which sets the loop condition on the device.  The host neither
// waits nor reads anything back.
// ---------------------------------------------------------------------------------------
// two internal streams per device to record the graph on: one for the prelude (when the
// caller's stream is not being captured itself) and one for the loop body.  Created on first
// use with this thread's capture mode relaxed, so that a first use inside the caller's own
// capture is legal; the mutex also serialises the recordings.
struct CaptureLanes {
    int device;
    cudaStream_t main, body;
};
constexpr int MAX_CAPTURE_DEVICES = 64;
std::mutex capture_mutex;
CaptureLanes capture_lanes[MAX_CAPTURE_DEVICES];
int n_capture_lanes = 0;

CaptureLanes *capture_lanes_for_current_device()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    for (int e = 0; e < n_capture_lanes; ++e)
        if (capture_lanes[e].device == dev) return &capture_lanes[e];
    if (n_capture_lanes == MAX_CAPTURE_DEVICES) return nullptr;
    CaptureLanes ln{dev, nullptr, nullptr};
    cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
    if (cudaThreadExchangeStreamCaptureMode(&mode) != cudaSuccess) return nullptr;
    bool ok = cudaStreamCreateWithFlags(&ln.main, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&ln.body, cudaStreamNonBlocking) == cudaSuccess;
    cudaThreadExchangeStreamCaptureMode(&mode);
    if (!ok) {
        if (ln.body) cudaStreamDestroy(ln.body);
        if (ln.main) cudaStreamDestroy(ln.main);
        return nullptr;
    }
    capture_lanes[n_capture_lanes] = ln;
    return &capture_lanes[n_capture_lanes++];
}

// Records the prelude and the WHILE node on `cap` (the caller's capturing stream, or an
// internal stream capturing into a fresh graph).
template <typename T>
int record_reinit_tol(T *F, int max_iters, double tol, double band, Ptr6<const T> d, TolWork<T> &w, const Grid &g,
                      int *status, double *history, cudaStream_t cap, cudaStream_t body_stream)
{
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t ndeps = 0;
    VSL_TRY(cudaStreamGetCaptureInfo(cap, &cs, nullptr, &graph, &deps, &edges, &ndeps));
    if (cs != cudaStreamCaptureStatusActive || graph == nullptr) return VSL_ERR_CUDA;
    cudaGraphConditionalHandle handle;
    VSL_TRY(cudaGraphConditionalHandleCreate(&handle, graph, 0, cudaGraphCondAssignDefault));
    // the FP32 band counter that the body's last stage leaves set (zeroed by the residual)
    unsigned *left_set = std::is_same<T, float>::value ? w.re.band.q.counter : nullptr;
    ResidualState rs{w.max_bits, w.ticket, status, history, left_set, tol, max_iters, 0, 1, handle};
    // prelude: counters, the classification (mask = F < 0 on entry), the input's residual
    VSL_TRY(cudaMemsetAsync(status, 0, 2 * sizeof(int), cap));
    VSL_TRY(cudaMemsetAsync(w.max_bits, 0, 2 * sizeof(unsigned long long), cap));
    if (int st = band_reset(w.re.band, cap)) return st;
    VSL_TRY(launch_classify<T>(F, d, w.re.flags, NodeList{nullptr, nullptr}, g, cap));
    VSL_TRY(launch_reinit_residual<T>(F, w.re.flags, d, g, band, rs, cap));
    // the WHILE node after the prelude
    VSL_TRY(cudaStreamGetCaptureInfo(cap, &cs, nullptr, &graph, &deps, &edges, &ndeps));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    VSL_TRY(cudaGraphAddNode(&node, graph, deps, edges, ndeps, &cp));
    VSL_TRY(cudaStreamUpdateCaptureDependencies(cap, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    // body (kernel nodes only): condition to 0 first (only a completed residual evaluation
    // continues the loop), one pseudo-step, the residual (counts the step, records it, sets
    // the condition, zeroes the band counter the next pseudo-step's first stage appends to)
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    VSL_TRY(cudaStreamBeginCaptureToGraph(body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int st = launch_condition_reset(handle, body_stream) == cudaSuccess ? VSL_OK : VSL_ERR_CUDA;
    if (st == VSL_OK) st = reinit_pseudo_step<T>(F, d, w.re, g, body_stream);
    rs.advance = 1;
    if (st == VSL_OK && launch_reinit_residual<T>(F, w.re.flags, d, g, band, rs, body_stream) != cudaSuccess)
        st = VSL_ERR_CUDA;
    cudaGraph_t out = nullptr;
    if (cudaStreamEndCapture(body_stream, &out) != cudaSuccess && st == VSL_OK) st = VSL_ERR_CUDA;
    return st;
}

template <typename T>
int op_reinit_tol(T *F, int max_iters, double tol, double band, const T *xpr, const T *xpl, const T *ypf,
                  const T *ypb, const T *zpu, const T *zpd, int rows, int cols, int pges, double dx, double dy,
                  double dz, int *status, double *history, void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F, xpr, xpl, ypf, ypb, zpu, zpd, status)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (max_iters < 0 || !(tol >= 0) || !(band > 0)) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_REINIT_TOL, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    TolWork<T> w = carve_tol<T>(b, g);
    Ptr6<const T> d = six(xpr, xpl, ypf, ypb, zpu, zpd);
    cudaStreamCaptureStatus cs;
    VSL_TRY(cudaStreamIsCapturing(s, &cs));
    std::lock_guard<std::mutex> lock(capture_mutex);
    CaptureLanes *ln = capture_lanes_for_current_device();
    if (ln == nullptr) return VSL_ERR_CUDA;
    if (cs == cudaStreamCaptureStatusActive)  // inside the caller's capture: add to its graph
        return record_reinit_tol<T>(F, max_iters, tol, band, d, w, g, status, history, s, ln->body);
    if (cs != cudaStreamCaptureStatusNone) return VSL_ERR_CUDA;
    // record a graph of its own, launch it on the caller's stream and release it (an
    // executable graph destroyed while in flight is freed once its launch completes)
    VSL_TRY(cudaStreamBeginCapture(ln->main, cudaStreamCaptureModeThreadLocal));
    int st = record_reinit_tol<T>(F, max_iters, tol, band, d, w, g, status, history, ln->main, ln->body);
    cudaGraph_t graph = nullptr;
    if (cudaStreamEndCapture(ln->main, &graph) != cudaSuccess && st == VSL_OK) st = VSL_ERR_CUDA;
    cudaGraphExec_t exec = nullptr;
    if (st == VSL_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) st = VSL_ERR_CUDA;
    if (st == VSL_OK && cudaGraphLaunch(exec, s) != cudaSuccess) st = VSL_ERR_CUDA;
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    return st;
}

// ---------------------------------------------------------------------------------------
// a batch of vesicle steps (FP32): the composite step of op_vesicle_step for every vesicle,
// with each RK stage of all the vesicles as one launch (launch_tiled_batch); the
// per-vesicle set-up passes (toolbox, extension velocity and crossing values, time step,
// setDistance, classification) stay per vesicle, spread over BATCH_LANES streams forked
// from and joined back into the caller's stream (parallel branches under stream capture).
// Vesicles are taken TILED_BATCH_MAX at a time.
// ---------------------------------------------------------------------------------------
constexpr int BATCH_LANES = 8;
struct BatchLanes {
    int device;
    cudaStream_t user;
    cudaStream_t lane[BATCH_LANES];
    cudaEvent_t fork, join[BATCH_LANES];
};
constexpr int MAX_BATCH_LANE_SETS = 64;
std::mutex batch_lane_mutex;
BatchLanes batch_lane_sets[MAX_BATCH_LANE_SETS];
int n_batch_lane_sets = 0;

// the lanes of (current device, caller stream), created on first use with this thread's
// capture mode relaxed; nullptr (everything on the caller's stream) when the pool is full or
// a creation fails
BatchLanes *batch_lanes(cudaStream_t s)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lock(batch_lane_mutex);
    for (int e = 0; e < n_batch_lane_sets; ++e)
        if (batch_lane_sets[e].device == dev && batch_lane_sets[e].user == s) return &batch_lane_sets[e];
    if (n_batch_lane_sets == MAX_BATCH_LANE_SETS) return nullptr;
    BatchLanes ln{};
    ln.device = dev;
    ln.user = s;
    cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
    if (cudaThreadExchangeStreamCaptureMode(&mode) != cudaSuccess) return nullptr;
    bool ok = cudaEventCreateWithFlags(&ln.fork, cudaEventDisableTiming) == cudaSuccess;
    for (int l = 0; l < BATCH_LANES && ok; ++l) {
        ok = cudaStreamCreateWithFlags(&ln.lane[l], cudaStreamNonBlocking) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&ln.join[l], cudaEventDisableTiming) == cudaSuccess;
    }
    cudaThreadExchangeStreamCaptureMode(&mode);
    if (!ok) {
        for (int l = 0; l < BATCH_LANES; ++l) {
            if (ln.join[l]) cudaEventDestroy(ln.join[l]);
            if (ln.lane[l]) cudaStreamDestroy(ln.lane[l]);
        }
        if (ln.fork) cudaEventDestroy(ln.fork);
        return nullptr;
    }
    batch_lane_sets[n_batch_lane_sets] = ln;
    return &batch_lane_sets[n_batch_lane_sets++];
}

// per-vesicle passes fanned out over the lanes: open() forks them from the caller's stream,
// lane(v) is vesicle v's stream, close() joins them back
struct Fan {
    BatchLanes *ln;
    cudaStream_t s;
    cudaError_t open()
    {
        if (!ln) return cudaSuccess;
        VSL_TRY_CUDA(cudaEventRecord(ln->fork, s));
        for (int l = 0; l < BATCH_LANES; ++l) VSL_TRY_CUDA(cudaStreamWaitEvent(ln->lane[l], ln->fork, 0));
        return cudaSuccess;
    }
    cudaStream_t lane(int v) const { return ln ? ln->lane[v % BATCH_LANES] : s; }
    cudaError_t close()
    {
        if (!ln) return cudaSuccess;
        for (int l = 0; l < BATCH_LANES; ++l) {
            VSL_TRY_CUDA(cudaEventRecord(ln->join[l], ln->lane[l]));
            VSL_TRY_CUDA(cudaStreamWaitEvent(s, ln->join[l], 0));
        }
        return cudaSuccess;
    }
};

struct BatchMember {
    Grid g;
    float *F;
    Ptr6<float> dist;
    double *info;
    StepWork<float> w;
    ReinitWork<float> adv, re;  // the advection and reinitialization views of w.ext
};

int check_vesicle(const vsl_vesicle_f32 &v)
{
    if (any_null(v.F, v.xpr, v.xpl, v.ypf, v.ypb, v.zpu, v.zpd, v.info)) return VSL_ERR_NULL;
    if (int st = check_grid(v.rows, v.cols, v.pges, v.dx, v.dy, v.dz)) return st;
    const Grid g = make_grid(v.rows, v.cols, v.pges, v.dx, v.dy, v.dz);
    return check_ws(VSL_OP_VESICLE_STEP, g, sizeof(float), v.workspace, v.workspace_bytes);
}

int batch_chunk(const vsl_vesicle_f32 *ves, int n, int ext_iters, int reinit_iters, double cfl, cudaStream_t s)
{
    BatchMember m[TILED_BATCH_MAX];
    TiledStage st[TILED_BATCH_MAX];
    Grid grids[TILED_BATCH_MAX];
    for (int v = 0; v < n; ++v) {
        const vsl_vesicle_f32 &d = ves[v];
        BatchMember &b = m[v];
        b.g = grids[v] = make_grid(d.rows, d.cols, d.pges, d.dx, d.dy, d.dz);
        b.F = d.F;
        b.dist = Ptr6<float>{{d.xpr, d.xpl, d.ypf, d.ypb, d.zpu, d.zpd}};
        b.info = d.info;
        Bump bump(d.workspace);
        b.w = carve_step<float>(bump, b.g);
        b.adv = ReinitWork<float>{};
        b.adv.b = b.w.ext.b;
        b.adv.c = b.w.ext.c;
        b.adv.band = b.w.ext.band;
        b.re = b.adv;
        b.re.flags = b.w.ext.flags;
    }
    // per vesicle: toolbox (mean curvature, normals, area, volume), the extension's
    // velocity, classification and crossing values of the mean curvature, its shadow
    Fan fan{batch_lanes(s), s};
    VSL_TRY(fan.open());
    for (int v = 0; v < n; ++v) {
        BatchMember &b = m[v];
        const cudaStream_t s = fan.lane(v);
        const double ds = (b.g.dx + b.g.dy + b.g.dz) / 3;
        ToolboxOut<float> tb{};
        tb.f[4] = b.w.nrm.p[0];
        tb.f[5] = b.w.nrm.p[1];
        tb.f[6] = b.w.nrm.p[2];
        tb.f[14] = b.w.vn;
        int nb = 0;
        VSL_TRY(launch_toolbox<float>(b.F, tb, b.g, ds, b.w.red.partials, &nb, s));
        VSL_TRY(launch_sum_partials(b.w.red.partials, nb, 2, std::pow(ds, 3), b.info, s));
        const Ptr6<const float> d = cview(b.dist);
        if (int r = extend_setup<float>(b.F, d, b.w.ext, b.g, false, 1e-6, s)) return r;
        VSL_TRY(launch_crossing_mixed(b.w.vn, d, b.w.ext.cp64, b.w.ext.flagged, b.g, false, s));
        VSL_TRY(launch_shadow_init(b.w.vn, b.w.ext.sh[0], b.w.ext.flagged, s));
        if (int r = band_reset(b.w.ext.band, s)) return r;
    }
    VSL_TRY(fan.close());
    // extension of the normal speed: each stage of all vesicles as one launch
    for (int it = 0; it < ext_iters; ++it) {
        for (int stage = 0; stage < 3; ++stage) {
            for (int v = 0; v < n; ++v) {
                BatchMember &b = m[v];
                ExtendWork<float> &e = b.w.ext;
                float *in = stage == 0 ? b.w.vn : (stage == 1 ? e.b : e.c);
                float *out = stage == 0 ? e.b : (stage == 1 ? e.c : b.w.vn);
                double *s_in = e.sh[stage], *s_out = e.sh[stage == 2 ? 0 : stage + 1];
                st[v] = TiledStage{in, b.w.vn, out, e.flags, cview(b.dist),
                                   BandShadow{s_in, e.sh[0], s_out, cview(e.cp64)}, cview3(e.v), nullptr, nullptr,
                                   e.band.q, e.flagged, stage, e.band.seq++};
            }
            VSL_TRY(launch_tiled_batch(1, false, st, grids, n, s));
        }
    }
    // per vesicle: dt = cfl * Ds / max |Vn| over |F| < 2 Ds
    VSL_TRY(fan.open());
    for (int v = 0; v < n; ++v) {
        BatchMember &b = m[v];
        const cudaStream_t s = fan.lane(v);
        const double ds = (b.g.dx + b.g.dy + b.g.dz) / 3;
        int nb = 0;
        VSL_TRY(launch_band_maxabs<float>(b.w.vn, b.F, 2 * ds, b.g, b.w.red.partials, &nb, s));
        VSL_TRY(launch_time_step(b.w.red.partials, nb, cfl * ds, b.info + 2, b.info + 3, s));
    }
    VSL_TRY(fan.close());
    // one WENO5 TVD-RK3 advection step along Vn * N
    for (int stage = 0; stage < 3; ++stage) {
        for (int v = 0; v < n; ++v) {
            BatchMember &b = m[v];
            float *in = stage == 0 ? b.F : (stage == 1 ? b.adv.b : b.adv.c);
            float *out = stage == 0 ? b.adv.b : (stage == 1 ? b.adv.c : b.F);
            st[v] = TiledStage{in, b.F, out, nullptr, Ptr6<const float>{}, BandShadow{}, cview3(b.w.nrm), b.w.vn,
                               b.info + 2, b.adv.band.q, NodeList{nullptr, nullptr}, stage, b.adv.band.seq++};
        }
        VSL_TRY(launch_tiled_batch(2, false, st, grids, n, s));
    }
    // per vesicle: setDistance and the classification of the reinitialization
    VSL_TRY(fan.open());
    for (int v = 0; v < n; ++v) {
        BatchMember &b = m[v];
        const cudaStream_t s = fan.lane(v);
        VSL_TRY(launch_set_distance<float>(b.F, b.dist, b.g, true, b.w.edges, s));
        VSL_TRY(launch_classify<float>(b.F, cview(b.dist), b.re.flags, NodeList{nullptr, nullptr}, b.g, s));
        if (int r = band_reset(b.re.band, s)) return r;
    }
    VSL_TRY(fan.close());
    for (int it = 0; it < reinit_iters; ++it) {
        for (int stage = 0; stage < 3; ++stage) {
            for (int v = 0; v < n; ++v) {
                BatchMember &b = m[v];
                float *in = stage == 0 ? b.F : (stage == 1 ? b.re.b : b.re.c);
                float *out = stage == 0 ? b.re.b : (stage == 1 ? b.re.c : b.F);
                st[v] = TiledStage{in, b.F, out, b.re.flags, cview(b.dist), BandShadow{}, Ptr3<const float>{},
                                   nullptr, nullptr, b.re.band.q, NodeList{nullptr, nullptr}, stage,
                                   b.re.band.seq++};
            }
            VSL_TRY(launch_tiled_batch(0, false, st, grids, n, s));
        }
    }
    return VSL_OK;
}

int op_vesicle_step_batch(const vsl_vesicle_f32 *ves, int count, int ext_iters, int reinit_iters, double cfl,
                          cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (ves == nullptr && count > 0) return VSL_ERR_NULL;
    if (count < 0 || ext_iters < 0 || reinit_iters < 0 || !(cfl > 0)) return VSL_ERR_VALUE;
    for (int v = 0; v < count; ++v)
        if (int st = check_vesicle(ves[v])) return st;
    for (int v0 = 0; v0 < count; v0 += TILED_BATCH_MAX)
        if (int st = batch_chunk(ves + v0, std::min(TILED_BATCH_MAX, count - v0), ext_iters, reinit_iters, cfl, s))
            return st;
    return VSL_OK;
}

// A batch of WENO5RK3Reinitialization calls (op_reinit_weno5 per member): each member's
// classification on its lane, then each RK stage of all members as one launch
int check_reinit_member(const vsl_reinit_f32 &r)
{
    if (any_null(r.F, r.xpr, r.xpl, r.ypf, r.ypb, r.zpu, r.zpd)) return VSL_ERR_NULL;
    if (int st = check_grid(r.rows, r.cols, r.pges, r.dx, r.dy, r.dz)) return st;
    const Grid g = make_grid(r.rows, r.cols, r.pges, r.dx, r.dy, r.dz);
    return check_ws(VSL_OP_REINIT_WENO5, g, sizeof(float), r.workspace, r.workspace_bytes);
}

int reinit_batch_chunk(const vsl_reinit_f32 *mem, int n, int iteration, cudaStream_t s)
{
    ReinitWork<float> w[TILED_BATCH_MAX];
    Ptr6<const float> d[TILED_BATCH_MAX];
    TiledStage st[TILED_BATCH_MAX];
    Grid grids[TILED_BATCH_MAX];
    for (int v = 0; v < n; ++v) {
        const vsl_reinit_f32 &r = mem[v];
        grids[v] = make_grid(r.rows, r.cols, r.pges, r.dx, r.dy, r.dz);
        Bump bump(r.workspace);
        w[v] = carve_reinit<float>(bump, grids[v], false);
        d[v] = six(r.xpr, r.xpl, r.ypf, r.ypb, r.zpu, r.zpd);
    }
    Fan fan{batch_lanes(s), s};
    VSL_TRY(fan.open());
    for (int v = 0; v < n; ++v) {
        const cudaStream_t ls = fan.lane(v);
        VSL_TRY(launch_classify<float>(mem[v].F, d[v], w[v].flags, NodeList{nullptr, nullptr}, grids[v], ls));
        if (int r = band_reset(w[v].band, ls)) return r;
    }
    VSL_TRY(fan.close());
    for (int it = 0; it < iteration; ++it) {
        for (int stage = 0; stage < 3; ++stage) {
            for (int v = 0; v < n; ++v) {
                float *F = mem[v].F;
                float *in = stage == 0 ? F : (stage == 1 ? w[v].b : w[v].c);
                float *out = stage == 0 ? w[v].b : (stage == 1 ? w[v].c : F);
                st[v] = TiledStage{in, F, out, w[v].flags, d[v], BandShadow{}, Ptr3<const float>{}, nullptr, nullptr,
                                   w[v].band.q, NodeList{nullptr, nullptr}, stage, w[v].band.seq++};
            }
            VSL_TRY(launch_tiled_batch(0, false, st, grids, n, s));
        }
    }
    return VSL_OK;
}

// A batch of WENO5RK3Extend calls (op_extend_weno5 per member): each member's velocity,
// classification, FP64 crossing values and shadow on its lane, then each RK stage of all
// members as one launch (the extension's band blocks inside it, per member)
int check_extend_member(const vsl_extend_f32 &e)
{
    if (any_null(e.C, e.F, e.xpr, e.xpl, e.ypf, e.ypb, e.zpu, e.zpd)) return VSL_ERR_NULL;
    if (int st = check_grid(e.rows, e.cols, e.pges, e.dx, e.dy, e.dz)) return st;
    const Grid g = make_grid(e.rows, e.cols, e.pges, e.dx, e.dy, e.dz);
    return check_ws(VSL_OP_EXTEND_WENO5, g, sizeof(float), e.workspace, e.workspace_bytes);
}

int extend_batch_chunk(const vsl_extend_f32 *mem, int n, int iteration, cudaStream_t s)
{
    ExtendWork<float> w[TILED_BATCH_MAX];
    Ptr6<const float> d[TILED_BATCH_MAX];
    TiledStage st[TILED_BATCH_MAX];
    Grid grids[TILED_BATCH_MAX];
    for (int v = 0; v < n; ++v) {
        const vsl_extend_f32 &e = mem[v];
        grids[v] = make_grid(e.rows, e.cols, e.pges, e.dx, e.dy, e.dz);
        Bump bump(e.workspace);
        w[v] = carve_extend<float>(bump, grids[v], false);
        d[v] = six(e.xpr, e.xpl, e.ypf, e.ypb, e.zpu, e.zpd);
    }
    Fan fan{batch_lanes(s), s};
    VSL_TRY(fan.open());
    for (int v = 0; v < n; ++v) {
        const cudaStream_t ls = fan.lane(v);
        ExtendWork<float> &e = w[v];
        if (int r = extend_setup<float>(mem[v].F, d[v], e, grids[v], false, 1e-6, ls)) return r;
        VSL_TRY(launch_crossing_mixed(mem[v].C, d[v], e.cp64, e.flagged, grids[v], false, ls));
        VSL_TRY(launch_shadow_init(mem[v].C, e.sh[0], e.flagged, ls));
        if (int r = band_reset(e.band, ls)) return r;
    }
    VSL_TRY(fan.close());
    for (int it = 0; it < iteration; ++it) {
        for (int stage = 0; stage < 3; ++stage) {
            for (int v = 0; v < n; ++v) {
                ExtendWork<float> &e = w[v];
                float *C = mem[v].C;
                float *in = stage == 0 ? C : (stage == 1 ? e.b : e.c);
                float *out = stage == 0 ? e.b : (stage == 1 ? e.c : C);
                double *s_out = e.sh[stage == 2 ? 0 : stage + 1];
                st[v] = TiledStage{in, C, out, e.flags, d[v], BandShadow{e.sh[stage], e.sh[0], s_out, cview(e.cp64)},
                                   cview3(e.v), nullptr, nullptr, e.band.q, e.flagged, stage, e.band.seq++};
            }
            VSL_TRY(launch_tiled_batch(1, false, st, grids, n, s));
        }
    }
    return VSL_OK;
}

int op_extend_batch(const vsl_extend_f32 *mem, int count, int iteration, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (mem == nullptr && count > 0) return VSL_ERR_NULL;
    if (count < 0 || iteration < 0) return VSL_ERR_VALUE;
    for (int v = 0; v < count; ++v)
        if (int st = check_extend_member(mem[v])) return st;
    for (int v0 = 0; v0 < count; v0 += TILED_BATCH_MAX)
        if (int st = extend_batch_chunk(mem + v0, std::min(TILED_BATCH_MAX, count - v0), iteration, s)) return st;
    return VSL_OK;
}

// A batch of WENO5 RK3 advections (op_advection per member): each RK stage of all members as
// one launch, `steps` steps of each member's device time step
int check_advect_member(const vsl_advect_f32 &a)
{
    if (any_null(a.F, a.vx, a.vy, a.vz, a.dt)) return VSL_ERR_NULL;
    if (int st = check_grid(a.rows, a.cols, a.pges, a.dx, a.dy, a.dz)) return st;
    const Grid g = make_grid(a.rows, a.cols, a.pges, a.dx, a.dy, a.dz);
    return check_ws(VSL_OP_ADVECTION, g, sizeof(float), a.workspace, a.workspace_bytes);
}

int advect_batch_chunk(const vsl_advect_f32 *mem, int n, int steps, cudaStream_t s)
{
    ReinitWork<float> w[TILED_BATCH_MAX];
    TiledStage st[TILED_BATCH_MAX];
    Grid grids[TILED_BATCH_MAX];
    for (int v = 0; v < n; ++v) {
        const vsl_advect_f32 &a = mem[v];
        grids[v] = make_grid(a.rows, a.cols, a.pges, a.dx, a.dy, a.dz);
        Bump bump(a.workspace);
        w[v] = carve_reinit<float>(bump, grids[v], false);
    }
    for (int it = 0; it < steps; ++it) {
        for (int stage = 0; stage < 3; ++stage) {
            for (int v = 0; v < n; ++v) {
                const vsl_advect_f32 &a = mem[v];
                float *in = stage == 0 ? a.F : (stage == 1 ? w[v].b : w[v].c);
                float *out = stage == 0 ? w[v].b : (stage == 1 ? w[v].c : a.F);
                st[v] = TiledStage{in, a.F, out, nullptr, Ptr6<const float>{}, BandShadow{},
                                   Ptr3<const float>{{a.vx, a.vy, a.vz}}, nullptr, a.dt, w[v].band.q,
                                   NodeList{nullptr, nullptr}, stage, w[v].band.seq++};
            }
            VSL_TRY(launch_tiled_batch(2, false, st, grids, n, s));
        }
    }
    return VSL_OK;
}

int op_advect_batch(const vsl_advect_f32 *mem, int count, int steps, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (mem == nullptr && count > 0) return VSL_ERR_NULL;
    if (count < 0 || steps < 0) return VSL_ERR_VALUE;
    for (int v = 0; v < count; ++v)
        if (int st = check_advect_member(mem[v])) return st;
    for (int v0 = 0; v0 < count; v0 += TILED_BATCH_MAX)
        if (int st = advect_batch_chunk(mem + v0, std::min(TILED_BATCH_MAX, count - v0), steps, s)) return st;
    return VSL_OK;
}

// A batch of closest-point surface redistances (op_redistance per member, WENO5 or WENORK3
// form): the set-up passes and each extension loop's crossing values and shadow per member
// on its lane; each RK stage of the extensions and of the reinitialization of all members
// as one launch
int check_redistance_member(const vsl_redistance_f32 &r, int op)
{
    if (any_null(r.A, r.F)) return VSL_ERR_NULL;
    if (int st = check_grid(r.rows, r.cols, r.pges, r.dx, r.dy, r.dz)) return st;
    const Grid g = make_grid(r.rows, r.cols, r.pges, r.dx, r.dy, r.dz);
    return check_ws(op, g, sizeof(float), r.workspace, r.workspace_bytes);
}

int redistance_batch_chunk(const vsl_redistance_f32 *mem, int n, int iter1, int iter2, bool eno3, cudaStream_t s)
{
    RedistWork<float> w[TILED_BATCH_MAX];
    TiledStage st[TILED_BATCH_MAX];
    Grid grids[TILED_BATCH_MAX];
    float *src[TILED_BATCH_MAX];
    for (int v = 0; v < n; ++v) {
        const vsl_redistance_f32 &r = mem[v];
        grids[v] = make_grid(r.rows, r.cols, r.pges, r.dx, r.dy, r.dz);
        Bump bump(r.workspace);
        w[v] = carve_redist<float>(bump, grids[v]);
    }
    Fan fan{batch_lanes(s), s};
    // set-up (ClosetPointSurfaceRedistance.m:15-74): A's distances and classes, F's distances,
    // normals and classes
    VSL_TRY(fan.open());
    for (int v = 0; v < n; ++v) {
        const cudaStream_t ls = fan.lane(v);
        RedistWork<float> &rw = w[v];
        VSL_TRY(launch_set_distance<float>(mem[v].A, rw.re.dist, grids[v], !eno3, rw.re.edges, ls));
        VSL_TRY(launch_classify<float>(mem[v].A, cview(rw.re.dist), rw.re.flags, NodeList{nullptr, nullptr},
                                       grids[v], ls));
        VSL_TRY(launch_set_distance<float>(mem[v].F, rw.ext.dist, grids[v], !eno3, rw.ext.edges, ls));
        if (int r = extend_setup<float>(mem[v].F, cview(rw.ext.dist), rw.ext, grids[v], eno3, 1e-14, ls)) return r;
        if (int r = band_reset(rw.re.band, ls)) return r;
    }
    VSL_TRY(fan.close());
    // iter2 extension pseudo-steps of every member's src[v] off F (extend_loop per member)
    auto extend_all = [&]() -> int {
        VSL_TRY(fan.open());
        for (int v = 0; v < n; ++v) {
            const cudaStream_t ls = fan.lane(v);
            ExtendWork<float> &e = w[v].ext;
            VSL_TRY(launch_crossing_mixed(src[v], cview(e.dist), e.cp64, e.flagged, grids[v], eno3, ls));
            VSL_TRY(launch_shadow_init(src[v], e.sh[0], e.flagged, ls));
            if (int r = band_reset(e.band, ls)) return r;
        }
        VSL_TRY(fan.close());
        for (int it = 0; it < iter2; ++it) {
            for (int stage = 0; stage < 3; ++stage) {
                for (int v = 0; v < n; ++v) {
                    ExtendWork<float> &e = w[v].ext;
                    float *C = src[v];
                    float *in = stage == 0 ? C : (stage == 1 ? e.b : e.c);
                    float *out = stage == 0 ? e.b : (stage == 1 ? e.c : C);
                    double *s_out = e.sh[stage == 2 ? 0 : stage + 1];
                    st[v] = TiledStage{in, C, out, e.flags, cview(e.dist),
                                       BandShadow{e.sh[stage], e.sh[0], s_out, cview(e.cp64)}, cview3(e.v), nullptr,
                                       nullptr, e.band.q, e.flagged, stage, e.band.seq++};
                }
                VSL_TRY(launch_tiled_batch(1, eno3, st, grids, n, s));
            }
        }
        return VSL_OK;
    };
    // one reinitialization stage of every member: stage input src[v] into out(v)
    auto reinit_all = [&](int stage) -> int {
        for (int v = 0; v < n; ++v) {
            ReinitWork<float> &re = w[v].re;
            float *A = mem[v].A;
            float *out = stage == 0 ? re.b : (stage == 1 ? re.c : A);
            st[v] = TiledStage{src[v], A, out, re.flags, cview(re.dist), BandShadow{}, Ptr3<const float>{}, nullptr,
                               nullptr, re.band.q, NodeList{nullptr, nullptr}, stage, re.band.seq++};
        }
        VSL_TRY(launch_tiled_batch(0, eno3, st, grids, n, s));
        return VSL_OK;
    };
    for (int it = 0; it < iter1; ++it) {
        for (int stage = 0; stage < 3; ++stage) {
            for (int v = 0; v < n; ++v)
                src[v] = stage == 0 ? mem[v].A : (stage == 1 ? w[v].re.b : w[v].re.c);
            if (int r = extend_all()) return r;
            if (int r = reinit_all(stage)) return r;
        }
    }
    for (int v = 0; v < n; ++v) src[v] = mem[v].A;
    return extend_all();
}

int op_redistance_batch(const vsl_redistance_f32 *mem, int count, int iter1, int iter2, bool eno3, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (mem == nullptr && count > 0) return VSL_ERR_NULL;
    if (count < 0 || iter1 < 0 || iter2 < 0) return VSL_ERR_VALUE;
    const int op = eno3 ? VSL_OP_SURFACE_REDISTANCE_ENO3 : VSL_OP_SURFACE_REDISTANCE;
    for (int v = 0; v < count; ++v)
        if (int st = check_redistance_member(mem[v], op)) return st;
    for (int v0 = 0; v0 < count; v0 += TILED_BATCH_MAX)
        if (int st = redistance_batch_chunk(mem + v0, std::min(TILED_BATCH_MAX, count - v0), iter1, iter2, eno3, s))
            return st;
    return VSL_OK;
}

int op_reinit_batch(const vsl_reinit_f32 *mem, int count, int iteration, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (mem == nullptr && count > 0) return VSL_ERR_NULL;
    if (count < 0 || iteration < 0) return VSL_ERR_VALUE;
    for (int v = 0; v < count; ++v)
        if (int st = check_reinit_member(mem[v])) return st;
    for (int v0 = 0; v0 < count; v0 += TILED_BATCH_MAX)
        if (int st = reinit_batch_chunk(mem + v0, std::min(TILED_BATCH_MAX, count - v0), iteration, s)) return st;
    return VSL_OK;
}

// ---------------------------------------------------------------------------------------
// ENORK2 (ENORK2Reinitialization.m:3-45, ENORK2Extend.m:9-81)
// ---------------------------------------------------------------------------------------

// the FP32 reinitialization workspace's band storage as a node list (the FP64 form has none)
template <typename T> NodeList band_list(ReinitWork<T> &w) { return NodeList{w.band.q.queue, w.band.q.counter}; }

// one ENORK2 reinitialization stage; the FP32 form runs the tiled kernel on the uniform
// nodes and the per-node code on the flagged list (from the classification) beside it
template <typename T>
int enork2_reinit_stage(const T *in, const T *n_in, T *out, ReinitWork<T> &w, Ptr6<const T> d, const Grid &g,
                        int stage, cudaStream_t s)
{
    if constexpr (std::is_same<T, float>::value) {
        VSL_TRY(tiled(4, false, w.band, in, n_in, out, w.flags, d, BandShadow{}, Ptr3<const float>{}, nullptr,
                      nullptr, stage, g, s, band_list(w)));
        return VSL_OK;
    } else {
        VSL_TRY(launch_enork2_reinit_stage<T>(in, n_in, out, w.flags, d, g, stage, s));
        return VSL_OK;
    }
}

template <typename T>
int op_reinit_enork2(T *F, int iteration, int rows, int cols, int pges, double dx, double dy, double dz, void *ws,
                     size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (iteration < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_REINIT_ENORK2, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    ReinitWork<T> w = carve_reinit<T>(b, g, true);
    VSL_TRY(launch_set_distance_eno2<T>(F, w.dist, g, w.edges, s));
    const Ptr6<const T> d = cview(w.dist);
    VSL_TRY(launch_classify<T>(F, d, w.flags, band_list(w), g, s));
    for (int it = 0; it < iteration; ++it) {
        if (int st = enork2_reinit_stage<T>(F, F, w.b, w, d, g, 0, s)) return st;
        if (int st = enork2_reinit_stage<T>(w.b, F, F, w, d, g, 1, s)) return st;
    }
    return VSL_OK;
}

// crossing values of C, then `iters` Heun RK2 extension steps of C in place
template <typename T>
int enork2_extend_loop(T *C, int iters, Ptr6<const T> d, ExtendWork<T> &w, const Grid &g, cudaStream_t s)
{
    const Ptr3<const T> v = cview3(w.v);
    if constexpr (std::is_same<T, float>::value) {
        // tiled uniform nodes, the flagged list on the per-node code beside them with the FP64
        // crossing values and shadow of C
        VSL_TRY(launch_enork2_crossing_mixed(C, d, w.cp64, w.flagged, g, s));
        VSL_TRY(launch_shadow_init(C, w.sh[0], w.flagged, s));
        const Ptr6<const double> cp = cview(w.cp64);
        for (int it = 0; it < iters; ++it) {
            VSL_TRY(tiled(3, false, w.band, C, C, w.b, w.flags, d, BandShadow{w.sh[0], w.sh[0], w.sh[1], cp}, v,
                          nullptr, nullptr, 0, g, s, w.flagged));
            VSL_TRY(tiled(3, false, w.band, w.b, C, C, w.flags, d, BandShadow{w.sh[1], w.sh[0], w.sh[0], cp}, v,
                          nullptr, nullptr, 1, g, s, w.flagged));
        }
        return VSL_OK;
    } else {
        VSL_TRY(launch_enork2_crossing<T>(C, d, w.cp, w.flagged, g, s));
        const Ptr6<const T> cp = cview(w.cp);
        for (int it = 0; it < iters; ++it) {
            VSL_TRY(launch_enork2_extend_stage<T>(C, C, w.b, w.flags, d, cp, v, g, 0, s));
            VSL_TRY(launch_enork2_extend_stage<T>(w.b, C, C, w.flags, d, cp, v, g, 1, s));
        }
        return VSL_OK;
    }
}

template <typename T>
int op_extend_enork2(T *C, int iteration, const T *F, int rows, int cols, int pges, double dx, double dy, double dz,
                     void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(C, F)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (iteration < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_EXTEND_ENORK2, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    ExtendWork<T> w = carve_extend<T>(b, g, true);
    VSL_TRY(launch_set_distance_eno2<T>(F, w.dist, g, w.edges, s));
    const Ptr6<const T> d = cview(w.dist);
    VSL_TRY(launch_enork2_velocity<T>(F, d, w.v, g, 1e-6, s));
    VSL_TRY(launch_classify<T>(F, d, w.flags, w.flagged, g, s));
    return enork2_extend_loop<T>(C, iteration, d, w, g, s);
}

// ENORK2ClosetPointSurfaceRedistance.m:4-128
template <typename T>
int op_redistance_enork2(T *A, int iter1, int iter2, const T *F, int rows, int cols, int pges, double dx, double dy,
                         double dz, void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(A, F)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (iter1 < 0 || iter2 < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_SURFACE_REDISTANCE_ENORK2, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    RedistWork<T> w = carve_redist<T>(b, g);
    // A's distances, mask and pseudo time step (reinitialization)
    VSL_TRY(launch_set_distance_eno2<T>(A, w.re.dist, g, w.re.edges, s));
    const Ptr6<const T> dA = cview(w.re.dist);
    VSL_TRY(launch_classify<T>(A, dA, w.re.flags, band_list(w.re), g, s));
    // F's distances, normals (floor 1e-14) and pseudo time step (extensions)
    VSL_TRY(launch_set_distance_eno2<T>(F, w.ext.dist, g, w.ext.edges, s));
    const Ptr6<const T> dF = cview(w.ext.dist);
    VSL_TRY(launch_enork2_velocity<T>(F, dF, w.ext.v, g, 1e-14, s));
    VSL_TRY(launch_classify<T>(F, dF, w.ext.flags, w.ext.flagged, g, s));
    T *t = w.re.b;
    for (int it = 0; it < iter1; ++it) {
        if (int st = enork2_extend_loop<T>(A, iter2, dF, w.ext, g, s)) return st;
        if (int st = enork2_reinit_stage<T>(A, A, t, w.re, dA, g, 0, s)) return st;
        if (int st = enork2_extend_loop<T>(t, iter2, dF, w.ext, g, s)) return st;
        if (int st = enork2_reinit_stage<T>(t, A, A, w.re, dA, g, 2, s)) return st;
    }
    return enork2_extend_loop<T>(A, iter2, dF, w.ext, g, s);
}

// ---------------------------------------------------------------------------------------
// GD3.Laplacian, GD3.smoothGMRES / smoothFFT and the relaxation step of the vesicle driver
// (p00_test_singlephase_relax.m:60-196)
// ---------------------------------------------------------------------------------------

template <typename T>
int op_laplacian(const T *f, T *out, int rows, int cols, int pges, double dx, double dy, double dz, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(f, out)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    VSL_TRY(launch_laplacian<T>(f, out, make_grid(rows, cols, pges, dx, dy, dz), s));
    return VSL_OK;
}

template <typename T>
int op_gradient(const T *f, T *fx, T *fy, T *fz, int rows, int cols, int pges, double dx, double dy, double dz,
                cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(f, fx, fy, fz)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    VSL_TRY(launch_gradient<T>(f, fx, fy, fz, make_grid(rows, cols, pges, dx, dy, dz), s));
    return VSL_OK;
}

template <typename T>
int op_smooth(const T *rhs, T *out, const double *dt, double alpha, int exact, int rows, int cols, int pges, double dx,
              double dy, double dz, void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(rhs, out, dt)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (!(alpha >= 0)) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_SMOOTH, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    SpecWork<T> sp = carve_spec<T>(b, g);
    if (sp.work_bytes == 0 && sp.work == nullptr) return VSL_ERR_CUDA;
    return launch_smooth_bilaplacian<T>(rhs, out, dt, alpha, exact != 0, g, sp.spec, sp.work, sp.work_bytes, s);
}

// C extended off the zero set of F by WENORK3Extend (cubic distances of F) or ENORK2Extend
// (quadratic distances of F), in place
template <typename T>
int extend_eno3_inplace(T *C, int iters, const T *F, ExtendWork<T> &w, const Grid &g, cudaStream_t s)
{
    VSL_TRY(launch_set_distance<T>(F, w.dist, g, false, w.edges, s));
    const Ptr6<const T> d = cview(w.dist);
    if (int st = extend_setup<T>(F, d, w, g, true, 1e-6, s)) return st;
    return extend_loop<T>(C, iters, d, w, g, true, s);
}

template <typename T>
int extend_enork2_inplace(T *C, int iters, const T *F, ExtendWork<T> &w, const Grid &g, cudaStream_t s)
{
    VSL_TRY(launch_set_distance_eno2<T>(F, w.dist, g, w.edges, s));
    const Ptr6<const T> d = cview(w.dist);
    VSL_TRY(launch_enork2_velocity<T>(F, d, w.v, g, 1e-6, s));
    VSL_TRY(launch_classify<T>(F, d, w.flags, w.flagged, g, s));
    return enork2_extend_loop<T>(C, iters, d, w, g, s);
}

template <typename T>
int op_relax_step(T *F, T *xpr, T *xpl, T *ypf, T *ypb, T *zpu, T *zpd, double A0, double V0, double kappa,
                  double spon_c, double cfl, double alpha, int ext_iters, int reinit_iters, double *info, int rows,
                  int cols, int pges, double dx, double dy, double dz, void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F, xpr, xpl, ypf, ypb, zpu, zpd, info)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (!(cfl > 0) || !(alpha >= 0) || ext_iters < 0 || reinit_iters < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_RELAX_STEP, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    RelaxWork<T> w = carve_relax<T>(b, g);
    if (w.spec.work_bytes == 0 && w.spec.work == nullptr) return VSL_ERR_CUDA;
    const double ds = (dx + dy + dz) / 3, ds3 = std::pow(ds, 3);
    double *area_volume = info, *dt = info + 2, *vmax = info + 3, *mom = info + 4, *tp = info + 8, *ene = info + 10;
    int nb = 0;
    // calculus toolbox: mean and Gaussian curvature, |grad F|, DiracDelta; area and volume
    ToolboxOut<T> tb{};
    tb.f[3] = w.G;
    tb.f[14] = w.H;
    tb.f[15] = w.K;
    tb.f[17] = w.D;
    VSL_TRY(launch_toolbox<T>(F, tb, g, ds, w.red.partials, &nb, s));
    VSL_TRY(launch_sum_partials(w.red.partials, nb, 2, ds3, area_volume, s));
    // MeanCurvature = WENORK3Extend(MeanCurvature, ext_iters)
    if (int st = extend_eno3_inplace<T>(w.H, ext_iters, F, w.ext, g, s)) return st;
    // bending speed, ENORK2-extended
    VSL_TRY(launch_bending_speed<T>(w.H, w.K, w.nsb, g, kappa, spon_c, s));
    if (int st = extend_enork2_inplace<T>(w.nsb, ext_iters, F, w.ext, g, s)) return st;
    // Dt = cfl * Ds / max |NSB| over |F| < 2 Ds
    VSL_TRY(launch_band_maxabs<T>(w.nsb, F, 2 * ds, g, w.red.partials, &nb, s));
    VSL_TRY(launch_time_step(w.red.partials, nb, cfl * ds, dt, vmax, s));
    // tension and pressure
    VSL_TRY(launch_relax_moments<T>(F, w.H, w.nsb, w.D, w.G, 2 * ds, spon_c, false, g, w.red.partials, &nb, s));
    VSL_TRY(launch_sum_partials(w.red.partials, nb, 4, ds3, mom, s));
    VSL_TRY(launch_tension_pressure(mom, area_volume, dt, A0, V0, tp, s));
    // normal speed, smoothed by (I + alpha Dt L^2)^-1, ENORK2-extended
    VSL_TRY(launch_normal_speed<T>(w.H, w.nsb, w.G, tp, w.vn, g, s));
    if (int st = launch_smooth_bilaplacian<T>(w.vn, w.vn, dt, alpha, true, g, w.spec.spec, w.spec.work,
                                              w.spec.work_bytes, s))
        return st;
    if (int st = extend_enork2_inplace<T>(w.vn, ext_iters, F, w.ext, g, s)) return st;
    // F = F - Dt * v, setDistance
    VSL_TRY(launch_euler<T>(F, w.vn, dt, g, s));
    VSL_TRY(launch_set_distance<T>(F, Ptr6<T>{{xpr, xpl, ypf, ypb, zpu, zpd}}, g, true, w.edges, s));
    // the energy int (H - c0)^2 over the new band (the toolbox's DiracDelta, |grad F|)
    VSL_TRY(launch_relax_moments<T>(F, w.H, nullptr, w.D, w.G, 2 * ds, spon_c, true, g, w.red.partials, &nb, s));
    VSL_TRY(launch_sum_partials(w.red.partials, nb, 1, ds3, ene, s));
    if (reinit_iters > 0) {
        const Ptr6<const T> d = six<T>(xpr, xpl, ypf, ypb, zpu, zpd);
        VSL_TRY(launch_classify<T>(F, d, w.re.flags, NodeList{nullptr, nullptr}, g, s));
        return reinit_loop<T>(F, reinit_iters, d, w.re, g, false, s);
    }
    return VSL_OK;
}

// ---------------------------------------------------------------------------------------
// adjoints (no counterpart in the reference)
// ---------------------------------------------------------------------------------------

// Reverse sweep through the three stages of one RK3 step whose stage inputs are
// s0 (= the step input), s1, s2.  `jac(ps, lam, coef)` fills W (and the parameter
// adjoints) for the stage with input ps and output adjoint lam; on return lam holds the
// adjoint of s0.
template <typename T, typename Jac>
int rk3_reverse(const T *s0, const T *s1, const T *s2, T *lam, AdjWork<T> &w, const Grid &g, cudaStream_t s, Jac jac)
{
    // stage 2: out = 1/3 s0 + 2/3 (s2 - step(s2))
    VSL_TRY(jac(s2, lam, 2.0 / 3.0));
    VSL_TRY(launch_adj_axpy<T>(w.acc, lam, 1.0 / 3.0, true, g, s));
    VSL_TRY(launch_adj_gather<T>(w.W, lam, 2.0 / 3.0, nullptr, w.x, g, s));
    // stage 1: s2 = 3/4 s0 + 1/4 (s1 - step(s1))
    VSL_TRY(jac(s1, w.x, 0.25));
    VSL_TRY(launch_adj_axpy<T>(w.acc, w.x, 0.75, false, g, s));
    VSL_TRY(launch_adj_gather<T>(w.W, w.x, 0.25, nullptr, w.x, g, s));
    // stage 0: s1 = s0 - step(s0)
    VSL_TRY(jac(s0, w.x, 1.0));
    VSL_TRY(launch_adj_gather<T>(w.W, w.x, 1.0, w.acc, lam, g, s));
    return VSL_OK;
}

// stage inputs s1, s2 of one advection step from its input F, by the forward kernels
template <typename T>
int advect_stages(const T *F, Ptr3<const T> v, const double *dt, ReinitWork<T> &w, const Grid &g, cudaStream_t s)
{
    if constexpr (std::is_same<T, float>::value) {
        const Ptr6<const float> none6{};
        VSL_TRY(tiled(2, false, w.band, F, F, w.b, nullptr, none6, BandShadow{}, v, nullptr, dt, 0, g, s));
        VSL_TRY(tiled(2, false, w.band, w.b, F, w.c, nullptr, none6, BandShadow{}, v, nullptr, dt, 1, g, s));
    } else {
        VSL_TRY(launch_advect_stage<T>(F, F, w.b, v, nullptr, dt, g, 0, false, s));
        VSL_TRY(launch_advect_stage<T>(w.b, F, w.c, v, nullptr, dt, g, 1, false, s));
    }
    return VSL_OK;
}

// stage inputs s1, s2 of one reinitialization pseudo-step from its input F
template <typename T>
int reinit_stages(const T *F, Ptr6<const T> d, ReinitWork<T> &w, const Grid &g, cudaStream_t s)
{
    if constexpr (std::is_same<T, float>::value) {
        if (int st = band_reset(w.band, s)) return st;
        const Ptr3<const float> none3{};
        VSL_TRY(tiled(0, false, w.band, F, F, w.b, w.flags, d, BandShadow{}, none3, nullptr, nullptr, 0, g, s));
        VSL_TRY(tiled(0, false, w.band, w.b, F, w.c, w.flags, d, BandShadow{}, none3, nullptr, nullptr, 1, g, s));
    } else {
        VSL_TRY(launch_reinit_stage<T>(F, F, w.b, w.flags, d, g, 0, false, false, s));
        VSL_TRY(launch_reinit_stage<T>(w.b, F, w.c, w.flags, d, g, 1, false, false, s));
    }
    return VSL_OK;
}

template <typename T>
int op_advection_adjoint(const T *F, const T *vx, const T *vy, const T *vz, const double *dt, T *lam, T *gvx, T *gvy,
                         T *gvz, int rows, int cols, int pges, double dx, double dy, double dz, void *ws, size_t bytes,
                         cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F, vx, vy, vz, dt, lam, gvx, gvy, gvz)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_ADVECTION_ADJOINT, g, sizeof(T), ws, bytes)) return st;
    Bump b(ws);
    AdjWork<T> w = carve_adj<T>(b, g, false);
    const Ptr3<const T> v{{vx, vy, vz}};
    const Ptr3<T> gv{{gvx, gvy, gvz}};
    if (int st = advect_stages<T>(F, v, dt, w.re, g, s)) return st;
    auto jac = [&](const T *ps, const T *l, double coef) {
        return launch_adj_advect_jac<T>(ps, v, dt, l, coef, w.W, gv, g, s);
    };
    return rk3_reverse<T>(F, w.re.b, w.re.c, lam, w, g, s, jac);
}

template <typename T>
int op_reinit_adjoint(const T *F0, int iteration, T *lam, T *tape, int rows, int cols, int pges, double dx, double dy,
                      double dz, void *ws, size_t bytes, cudaStream_t s)
{
    VSL_RANGE(__func__);
    if (any_null(F0, lam, tape)) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    if (iteration < 0) return VSL_ERR_VALUE;
    Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    if (int st = check_ws(VSL_OP_REINIT_ADJOINT, g, sizeof(T), ws, bytes)) return st;
    if (iteration == 0) return VSL_OK;
    Bump b(ws);
    AdjWork<T> w = carve_adj<T>(b, g, true);
    ReinitWork<T> &re = w.re;
    // the forward set-up of WENO5RK3Reinitialization: distances of F0 (degree-5 roots),
    // classification, then the pseudo-step inputs phi^0 .. phi^{K-1} into the tape
    VSL_TRY(launch_set_distance<T>(F0, re.dist, g, true, re.edges, s));
    const Ptr6<const T> d = cview(re.dist);
    VSL_TRY(launch_classify<T>(F0, d, re.flags, NodeList{nullptr, nullptr}, g, s));
    const size_t field = sizeof(T) * (size_t)g.num;
    VSL_TRY(cudaMemcpyAsync(tape, F0, field, cudaMemcpyDeviceToDevice, s));
    for (int k = 1; k < iteration; ++k) {
        T *cur = tape + (size_t)k * g.num;
        VSL_TRY(cudaMemcpyAsync(cur, cur - g.num, field, cudaMemcpyDeviceToDevice, s));
        if (int st = reinit_loop<T>(cur, 1, d, re, g, false, s)) return st;
    }
    for (int q = 0; q < 6; ++q) VSL_TRY(cudaMemsetAsync(w.mu.p[q], 0, field, s));
    auto jac = [&](const T *ps, const T *l, double coef) {
        return launch_adj_reinit_jac<T>(ps, re.flags, d, l, coef, w.W, w.mu, w.band, g, s);
    };
    for (int k = iteration - 1; k >= 0; --k) {
        const T *phik = tape + (size_t)k * g.num;
        if (int st = reinit_stages<T>(phik, d, re, g, s)) return st;
        if (int st = rk3_reverse<T>(phik, re.b, re.c, lam, w, g, s, jac)) return st;
    }
    // the distances' dependence on F0
    VSL_TRY(launch_adj_dist_edges<T>(F0, re.edges, cview(w.mu), w.W, g, s));
    VSL_TRY(launch_adj_gather<T>(w.W, lam, 1.0, nullptr, lam, g, s));
    return VSL_OK;
}

}  // namespace
}  // namespace vsl

using namespace vsl;

extern "C" {

int vsl_vesicle_step_batch_f32(const vsl_vesicle_f32 *vesicles, int count, int ext_iters, int reinit_iters,
                               double cfl, vsl_stream_t stream)
{
    return op_vesicle_step_batch(vesicles, count, ext_iters, reinit_iters, cfl, reinterpret_cast<cudaStream_t>(stream));
}

int vsl_weno5_rk3_reinitialization_batch_f32(const vsl_reinit_f32 *members, int count, int iteration,
                                             vsl_stream_t stream)
{
    return op_reinit_batch(members, count, iteration, reinterpret_cast<cudaStream_t>(stream));
}

int vsl_weno5_rk3_extend_batch_f32(const vsl_extend_f32 *members, int count, int iteration, vsl_stream_t stream)
{
    return op_extend_batch(members, count, iteration, reinterpret_cast<cudaStream_t>(stream));
}

int vsl_weno5_rk3_advection_batch_f32(const vsl_advect_f32 *members, int count, int steps, vsl_stream_t stream)
{
    return op_advect_batch(members, count, steps, reinterpret_cast<cudaStream_t>(stream));
}

int vsl_weno5_rk3_surface_redistance_batch_f32(const vsl_redistance_f32 *members, int count, int iter1, int iter2,
                                               vsl_stream_t stream)
{
    return op_redistance_batch(members, count, iter1, iter2, false, reinterpret_cast<cudaStream_t>(stream));
}

int vsl_wenork3_surface_redistance_batch_f32(const vsl_redistance_f32 *members, int count, int iter1, int iter2,
                                             vsl_stream_t stream)
{
    return op_redistance_batch(members, count, iter1, iter2, true, reinterpret_cast<cudaStream_t>(stream));
}

const char *vsl_status_string(int status)
{
    switch (status) {
    case VSL_OK: return "ok";
    case VSL_ERR_NULL: return "null pointer argument";
    case VSL_ERR_SHAPE: return "bad grid shape";
    case VSL_ERR_VALUE: return "argument value out of range";
    case VSL_ERR_WORKSPACE: return "workspace missing, too small or not 256-byte aligned";
    case VSL_ERR_CUDA: return "CUDA launch failed";
    case VSL_ERR_OP: return "unknown operation";
    case VSL_ERR_SCRATCH_LIMIT: return "grid too large for the static scratch of a no-allocation entry point";
    default: return "unknown status";
    }
}

int vsl_version(void) { return 1; }

int vsl_set_tile_pages(int rows, int cols, int pges, int kind, int pages)
{
    return set_tile_pages(rows, cols, pges, kind, pages);
}

int vsl_set_plane_loads(int mode) { return set_plane_loads(mode); }

int vsl_plane_loads(void) { return get_plane_loads(); }

int vsl_tma_wait_timeouts(unsigned *count)
{
    if (count == nullptr) return VSL_ERR_NULL;
    return tma_timeouts(count) == cudaSuccess ? VSL_OK : VSL_ERR_CUDA;
}

int vsl_tile_pages(int rows, int cols, int pges, int kind)
{
    if (rows <= 0 || cols <= 0 || pges <= 0 || kind < 0 || kind > 4) return 0;
    return tile_pages(make_grid(rows, cols, pges, 1.0, 1.0, 1.0), kind);
}

size_t vsl_workspace_bytes(int op, int rows, int cols, int pges, int elem_bytes)
{
    if (rows <= 0 || cols <= 0 || pges <= 0) return 0;
    Grid g = make_grid(rows, cols, pges, 1.0, 1.0, 1.0);
    return measure(op, g, elem_bytes);
}

#define VSL_TYPED(SUF, T)                                                                                          \
    int vsl_set_distance_##SUF(const T *F, T *xpr, T *xpl, T *ypf, T *ypb, T *zpu, T *zpd, int rows, int cols,     \
                               int pges, double dx, double dy, double dz, void *ws, size_t bytes,                  \
                               vsl_stream_t stream)                                                                \
    {                                                                                                              \
        return op_set_distance<T>(F, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz, ws, bytes,        \
                                  stream);                                                                         \
    }                                                                                                              \
    int vsl_weno5_rk3_reinitialization_##SUF(T *F, int iteration, const T *xpr, const T *xpl, const T *ypf,        \
                                             const T *ypb, const T *zpu, const T *zpd, int rows, int cols,         \
                                             int pges, double dx, double dy, double dz, void *ws, size_t bytes,    \
                                             vsl_stream_t stream)                                                  \
    {                                                                                                              \
        return op_reinit_weno5<T>(F, iteration, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz, ws,    \
                                  bytes, stream);                                                                  \
    }                                                                                                              \
    int vsl_weno5_rk3_reinitialization_tol_##SUF(T *F, int max_iters, double tol, double band, const T *xpr,       \
                                                 const T *xpl, const T *ypf, const T *ypb, const T *zpu,           \
                                                 const T *zpd, int rows, int cols, int pges, double dx, double dy, \
                                                 double dz, int *status, double *residual, void *ws, size_t bytes, \
                                                 vsl_stream_t stream)                                              \
    {                                                                                                              \
        return op_reinit_tol<T>(F, max_iters, tol, band, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy,   \
                                dz, status, residual, ws, bytes, stream);                                          \
    }                                                                                                              \
    int vsl_wenork3_reinitialization_##SUF(T *F, int iteration, int rows, int cols, int pges, double dx,           \
                                           double dy, double dz, void *ws, size_t bytes, vsl_stream_t stream)      \
    {                                                                                                              \
        return op_reinit_eno3<T>(F, iteration, rows, cols, pges, dx, dy, dz, ws, bytes, stream);                   \
    }                                                                                                              \
    int vsl_weno5_rk3_extend_##SUF(T *C, int iteration, const T *F, const T *xpr, const T *xpl, const T *ypf,      \
                                   const T *ypb, const T *zpu, const T *zpd, int rows, int cols, int pges,         \
                                   double dx, double dy, double dz, void *ws, size_t bytes, vsl_stream_t stream)   \
    {                                                                                                              \
        return op_extend_weno5<T>(C, iteration, F, xpr, xpl, ypf, ypb, zpu, zpd, rows, cols, pges, dx, dy, dz, ws, \
                                  bytes, stream);                                                                  \
    }                                                                                                              \
    int vsl_wenork3_extend_##SUF(T *C, int iteration, const T *F, int rows, int cols, int pges, double dx,         \
                                 double dy, double dz, void *ws, size_t bytes, vsl_stream_t stream)                \
    {                                                                                                              \
        return op_extend_eno3<T>(C, iteration, F, rows, cols, pges, dx, dy, dz, ws, bytes, stream);                \
    }                                                                                                              \
    int vsl_weno5_rk3_surface_redistance_##SUF(T *A, int iter1, int iter2, const T *F, int rows, int cols,         \
                                               int pges, double dx, double dy, double dz, void *ws, size_t bytes,  \
                                               vsl_stream_t stream)                                                \
    {                                                                                                              \
        return op_redistance<T>(A, iter1, iter2, F, rows, cols, pges, dx, dy, dz, false, ws, bytes, stream);       \
    }                                                                                                              \
    int vsl_wenork3_surface_redistance_##SUF(T *A, int iter1, int iter2, const T *F, int rows, int cols, int pges, \
                                             double dx, double dy, double dz, void *ws, size_t bytes,              \
                                             vsl_stream_t stream)                                                  \
    {                                                                                                              \
        return op_redistance<T>(A, iter1, iter2, F, rows, cols, pges, dx, dy, dz, true, ws, bytes, stream);        \
    }                                                                                                              \
    int vsl_area_volume_##SUF(const T *F, double *area_volume, int rows, int cols, int pges, double dx, double dy, \
                              double dz, void *ws, size_t bytes, vsl_stream_t stream)                              \
    {                                                                                                              \
        return op_area_volume<T>(F, area_volume, rows, cols, pges, dx, dy, dz, ws, bytes, stream);                 \
    }                                                                                                              \
    int vsl_weno5_rk3_advection_##SUF(T *F, const T *vx, const T *vy, const T *vz, const double *dt, int steps,    \
                                      int rows, int cols, int pges, double dx, double dy, double dz, void *ws,     \
                                      size_t bytes, vsl_stream_t stream)                                           \
    {                                                                                                              \
        return op_advection<T>(F, vx, vy, vz, dt, steps, rows, cols, pges, dx, dy, dz, ws, bytes, stream);         \
    }                                                                                                              \
    int vsl_vesicle_step_##SUF(T *F, T *xpr, T *xpl, T *ypf, T *ypb, T *zpu, T *zpd, int ext_iters,                \
                               int reinit_iters, double cfl, double *info, int rows, int cols, int pges,           \
                               double dx, double dy, double dz, void *ws, size_t bytes, vsl_stream_t stream)       \
    {                                                                                                              \
        return op_vesicle_step<T>(F, xpr, xpl, ypf, ypb, zpu, zpd, ext_iters, reinit_iters, cfl, info, rows, cols, \
                                  pges, dx, dy, dz, ws, bytes, stream);                                            \
    }                                                                                                              \
    int vsl_enork2_reinitialization_##SUF(T *F, int iteration, int rows, int cols, int pges, double dx, double dy,  \
                                          double dz, void *ws, size_t bytes, vsl_stream_t stream)                   \
    {                                                                                                              \
        return op_reinit_enork2<T>(F, iteration, rows, cols, pges, dx, dy, dz, ws, bytes, stream);                 \
    }                                                                                                              \
    int vsl_enork2_extend_##SUF(T *C, int iteration, const T *F, int rows, int cols, int pges, double dx,          \
                                double dy, double dz, void *ws, size_t bytes, vsl_stream_t stream)                 \
    {                                                                                                              \
        return op_extend_enork2<T>(C, iteration, F, rows, cols, pges, dx, dy, dz, ws, bytes, stream);              \
    }                                                                                                              \
    int vsl_enork2_surface_redistance_##SUF(T *A, int iter1, int iter2, const T *F, int rows, int cols, int pges,   \
                                            double dx, double dy, double dz, void *ws, size_t bytes,                \
                                            vsl_stream_t stream)                                                    \
    {                                                                                                              \
        return op_redistance_enork2<T>(A, iter1, iter2, F, rows, cols, pges, dx, dy, dz, ws, bytes, stream);        \
    }                                                                                                              \
    int vsl_laplacian_##SUF(const T *field, T *out, int rows, int cols, int pges, double dx, double dy, double dz, \
                            vsl_stream_t stream)                                                                   \
    {                                                                                                              \
        return op_laplacian<T>(field, out, rows, cols, pges, dx, dy, dz, stream);                                  \
    }                                                                                                              \
    int vsl_gradient_##SUF(const T *field, T *fx, T *fy, T *fz, int rows, int cols, int pges, double dx,          \
                           double dy, double dz, vsl_stream_t stream)                                              \
    {                                                                                                              \
        return op_gradient<T>(field, fx, fy, fz, rows, cols, pges, dx, dy, dz, stream);                            \
    }                                                                                                              \
    int vsl_smooth_bilaplacian_##SUF(const T *rhs, T *out, const double *dt, double alpha, int exact, int rows,    \
                                     int cols, int pges, double dx, double dy, double dz, void *ws, size_t bytes,  \
                                     vsl_stream_t stream)                                                          \
    {                                                                                                              \
        return op_smooth<T>(rhs, out, dt, alpha, exact, rows, cols, pges, dx, dy, dz, ws, bytes, stream);          \
    }                                                                                                              \
    int vsl_relax_step_##SUF(T *F, T *xpr, T *xpl, T *ypf, T *ypb, T *zpu, T *zpd, double A0, double V0,           \
                             double kappa, double spon_c, double cfl, double alpha, int ext_iters, int reinit_iters, \
                             double *info, int rows, int cols, int pges, double dx, double dy, double dz, void *ws, \
                             size_t bytes, vsl_stream_t stream)                                                    \
    {                                                                                                              \
        return op_relax_step<T>(F, xpr, xpl, ypf, ypb, zpu, zpd, A0, V0, kappa, spon_c, cfl, alpha, ext_iters,     \
                                reinit_iters, info, rows, cols, pges, dx, dy, dz, ws, bytes, stream);              \
    }                                                                                                              \
    int vsl_weno5_rk3_advection_adjoint_##SUF(const T *F, const T *vx, const T *vy, const T *vz, const double *dt, \
                                              T *lam, T *gvx, T *gvy, T *gvz, int rows, int cols, int pges,        \
                                              double dx, double dy, double dz, void *ws, size_t bytes,             \
                                              vsl_stream_t stream)                                                 \
    {                                                                                                              \
        return op_advection_adjoint<T>(F, vx, vy, vz, dt, lam, gvx, gvy, gvz, rows, cols, pges, dx, dy, dz, ws,    \
                                       bytes, stream);                                                             \
    }                                                                                                              \
    int vsl_weno5_rk3_reinitialization_adjoint_##SUF(const T *F0, int iteration, T *lam, T *tape, int rows,        \
                                                     int cols, int pges, double dx, double dy, double dz,          \
                                                     void *ws, size_t bytes, vsl_stream_t stream)                  \
    {                                                                                                              \
        return op_reinit_adjoint<T>(F0, iteration, lam, tape, rows, cols, pges, dx, dy, dz, ws, bytes, stream);    \
    }                                                                                                              \
    int vsl_a_set_calculus_toolbox_##SUF(const T *A, const T *F, T *const *out, int rows, int cols, int pges,      \
                                         double dx, double dy, double dz, void *ws, size_t bytes,                  \
                                         vsl_stream_t stream)                                                      \
    {                                                                                                              \
        return op_aux_toolbox<T>(A, F, out, rows, cols, pges, dx, dy, dz, ws, bytes, stream);                      \
    }                                                                                                              \
    int vsl_masked_integral_##SUF(const T *F, const T *A, const T *f0, const T *f1, const T *f2,                   \
                                  const T *one_minus, double *result, int rows, int cols, int pges, double dx,     \
                                  double dy, double dz, void *ws, size_t bytes, vsl_stream_t stream)               \
    {                                                                                                              \
        return op_masked_integral<T>(F, A, f0, f1, f2, one_minus, result, rows, cols, pges, dx, dy, dz, ws, bytes, \
                                     stream);                                                                      \
    }

VSL_TYPED(f64, double)
VSL_TYPED(f32, float)

}  // extern "C"
