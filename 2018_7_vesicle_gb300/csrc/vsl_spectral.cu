// vsl_spectral.cu -- the bi-Laplacian smoothing of SD.GD3 (GD3.m:434-485) by FFT.
//
// smoothGMRES solves (I + alpha Dt L^2) x = rhs, L the 7-point Laplacian with periodic
// neighbours (GD3.m:110-189), by GMRES preconditioned with FFTs.  That operator is
// circulant, so the DFT diagonalises it exactly: its symbol is
//   1 + alpha Dt lambda^2,  lambda = sum_axis (2 cos(2 pi m / n) - 2) / h^2,
// and x = real(ifftn(fftn(rhs) ./ symbol)) is the system's solution, which the GMRES
// iteration approaches to its tolerance (1e-12).  smoothFFT applies the continuous symbol
// 1 + alpha Dt (kx^2 + ky^2 + kz^2)^2 with the wave numbers of GD3.m:195-207 (the
// fftshifted grid -n/2 : n/2-1, half-integers for odd n) in the same way.
//
// The transforms are cuFFT's complex-to-complex ones (a library FFT, as a GEMM would be
// cuBLAS), in place on a complex copy of rhs held in the caller's workspace; the plans
// are created once per grid shape and precision (the first call for a shape, or
// vsl_workspace_bytes, creates them), with cuFFT's work area also taken from the caller's
// workspace.  The scaling by 1/N of the inverse transform and the real part are fused
// into the last kernel.
#include <cufft.h>

#include <mutex>

#include "vsl_internal.h"

namespace vsl {
namespace {

template <typename T> struct Cx;
template <> struct Cx<double> {
    using type = cufftDoubleComplex;
    static constexpr cufftType kind = CUFFT_Z2Z;
};
template <> struct Cx<float> {
    using type = cufftComplex;
    static constexpr cufftType kind = CUFFT_C2C;
};

struct PlanEntry {
    int rows, cols, pges;
    bool fp64;
    cufftHandle plan;
    size_t work;
};
constexpr int MAX_PLANS = 64;
std::mutex plan_mutex;
PlanEntry plans[MAX_PLANS];
int n_plans = 0;

// the plan for a shape (created on first use, work area supplied per call)
template <typename T> int get_plan(const Grid &g, PlanEntry **out)
{
    const bool fp64 = sizeof(T) == 8;
    for (int e = 0; e < n_plans; ++e)
        if (plans[e].rows == g.rows && plans[e].cols == g.cols && plans[e].pges == g.pges && plans[e].fp64 == fp64) {
            *out = &plans[e];
            return VSL_OK;
        }
    if (n_plans == MAX_PLANS) return VSL_ERR_VALUE;
    PlanEntry p{g.rows, g.cols, g.pges, fp64, 0, 0};
    if (cufftCreate(&p.plan) != CUFFT_SUCCESS) return VSL_ERR_CUDA;
    if (cufftSetAutoAllocation(p.plan, 0) != CUFFT_SUCCESS ||
        cufftMakePlan3d(p.plan, g.pges, g.cols, g.rows, Cx<T>::kind, &p.work) != CUFFT_SUCCESS) {
        cufftDestroy(p.plan);
        return VSL_ERR_CUDA;
    }
    plans[n_plans] = p;
    *out = &plans[n_plans++];
    return VSL_OK;
}

template <typename T>
__global__ void k_to_complex(const T *__restrict__ in, typename Cx<T>::type *__restrict__ out, long long n)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        out[t].x = in[t];
        out[t].y = T(0);
    }
}

// MATLAB's fftshift of -n/2 : n/2-1 at transform index t (GD3.m:195-201)
__device__ __forceinline__ double shifted_wave(int t, int n)
{
    const int s = n / 2;
    const int u = ((t - s) % n + n) % n;
    return -0.5 * n + u;
}

// spec ./= 1 + alpha Dt symbol, symbol = lambda^2 (exact) or |k|^4 (continuous)
template <typename T>
__global__ void k_spectral_filter(typename Cx<T>::type *__restrict__ spec, Grid g, const double *__restrict__ dt,
                                  double alpha, int exact)
{
    const long long n = g.num;
    const double adt = alpha * __ldg(dt);
    const double two_pi = 6.283185307179586;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e / g.plane);
        const long long r = e - (long long)k * g.plane;
        const int j = (int)(r / g.rows);
        const int i = (int)(r - (long long)j * g.rows);
        double d;
        if (exact) {
            const double lam = (2 * cos(two_pi * j / g.cols) - 2) / (g.dx * g.dx) +
                               (2 * cos(two_pi * i / g.rows) - 2) / (g.dy * g.dy) +
                               (2 * cos(two_pi * k / g.pges) - 2) / (g.dz * g.dz);
            d = 1 + adt * (lam * lam);
        } else {
            const double kx = two_pi * shifted_wave(j, g.cols) / (g.cols * g.dx);
            const double ky = two_pi * shifted_wave(i, g.rows) / (g.rows * g.dy);
            const double kz = two_pi * shifted_wave(k, g.pges) / (g.pges * g.dz);
            const double s = kx * kx + ky * ky + kz * kz;
            d = 1 + adt * (s * s);
        }
        spec[e].x = (T)(spec[e].x / d);
        spec[e].y = (T)(spec[e].y / d);
    }
}

template <typename T>
__global__ void k_real_scaled(const typename Cx<T>::type *__restrict__ spec, T *__restrict__ out, long long n)
{
    const double inv = 1.0 / (double)n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        out[t] = (T)(spec[t].x * inv);
}

inline int spec_blocks()
{
    static int nb = 0;
    if (nb == 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        nb = (sms > 0 ? sms : 132) * 8;
    }
    return nb;
}

}  // namespace

template <typename T> size_t spectral_work_bytes(const Grid &g)
{
    std::lock_guard<std::mutex> lock(plan_mutex);
    PlanEntry *p = nullptr;
    if (get_plan<T>(g, &p) != VSL_OK) return 0;
    return p->work;
}

template <typename T>
int launch_smooth_bilaplacian(const T *rhs, T *out, const double *dt, double alpha, bool exact, const Grid &g,
                              void *spectrum, void *work, size_t work_bytes, cudaStream_t s)
{
    using C = typename Cx<T>::type;
    C *spec = static_cast<C *>(spectrum);
    k_to_complex<T><<<spec_blocks(), 256, 0, s>>>(rhs, spec, g.num);
    if (cudaGetLastError() != cudaSuccess) return VSL_ERR_CUDA;
    {
        std::lock_guard<std::mutex> lock(plan_mutex);
        PlanEntry *p = nullptr;
        if (int st = get_plan<T>(g, &p)) return st;
        if (p->work > work_bytes) return VSL_ERR_WORKSPACE;
        if (cufftSetStream(p->plan, s) != CUFFT_SUCCESS || cufftSetWorkArea(p->plan, work) != CUFFT_SUCCESS)
            return VSL_ERR_CUDA;
        cufftResult r;
        if constexpr (sizeof(T) == 8)
            r = cufftExecZ2Z(p->plan, spec, spec, CUFFT_FORWARD);
        else
            r = cufftExecC2C(p->plan, spec, spec, CUFFT_FORWARD);
        if (r != CUFFT_SUCCESS) return VSL_ERR_CUDA;
        k_spectral_filter<T><<<spec_blocks(), 256, 0, s>>>(spec, g, dt, alpha, exact ? 1 : 0);
        if (cudaGetLastError() != cudaSuccess) return VSL_ERR_CUDA;
        if constexpr (sizeof(T) == 8)
            r = cufftExecZ2Z(p->plan, spec, spec, CUFFT_INVERSE);
        else
            r = cufftExecC2C(p->plan, spec, spec, CUFFT_INVERSE);
        if (r != CUFFT_SUCCESS) return VSL_ERR_CUDA;
    }
    k_real_scaled<T><<<spec_blocks(), 256, 0, s>>>(spec, out, g.num);
    return cudaGetLastError() == cudaSuccess ? VSL_OK : VSL_ERR_CUDA;
}

template size_t spectral_work_bytes<double>(const Grid &);
template size_t spectral_work_bytes<float>(const Grid &);
template int launch_smooth_bilaplacian<double>(const double *, double *, const double *, double, bool, const Grid &,
                                               void *, void *, size_t, cudaStream_t);
template int launch_smooth_bilaplacian<float>(const float *, float *, const double *, double, bool, const Grid &,
                                              void *, void *, size_t, cudaStream_t);

}  // namespace vsl
