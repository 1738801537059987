// vsl_toolbox.cu -- the FP64 instantiation of the toolbox and band-maximum kernels
// (vsl_toolbox.cuh), the fixed-order sums of the block partials and the time step.
#include "vsl_toolbox.cuh"

namespace vsl {
namespace {

// result[q] = scale * sum_b partials[ncomp*b + q], fixed order (one block of 1024)
__global__ void __launch_bounds__(1024) k_sum_partials(const double *__restrict__ partials, int nblocks, int ncomp,
                                                       double scale, double *__restrict__ result)
{
    __shared__ double s[32];
    for (int q = 0; q < ncomp; ++q) {
        double acc = 0.0;
        // unrolled so that the loads are in flight together; the additions keep their order
#pragma unroll 8
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc += partials[(long long)ncomp * b + q];
        acc = warp_sum(acc);
        if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s[w];
            result[q] = tot * scale;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(1024) k_time_step(const double *__restrict__ partials, int nblocks, double cfl_ds,
                                                    double *__restrict__ dt, double *__restrict__ vmax)
{
    __shared__ double s[32];
    double m = 0.0;
#pragma unroll 8
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) m = fmax(m, partials[b]);
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, s[w]);
        if (vmax) *vmax = r;
        *dt = r > 0.0 ? cfl_ds / r : 0.0;
    }
}

}  // namespace

int toolbox_partial_blocks(const Grid &g)
{
    dim3 gr = node_grid(g);
    return (int)((long long)gr.x * gr.y * gr.z);
}

cudaError_t launch_sum_partials(const double *partials, int nblocks, int ncomp, double scale, double *result,
                                cudaStream_t s)
{
    k_sum_partials<<<1, 1024, 0, s>>>(partials, nblocks, ncomp, scale, result);
    return cudaGetLastError();
}

cudaError_t launch_time_step(const double *partials, int nblocks, double cfl_ds, double *dt, double *vmax,
                             cudaStream_t s)
{
    k_time_step<<<1, 1024, 0, s>>>(partials, nblocks, cfl_ds, dt, vmax);
    return cudaGetLastError();
}

template cudaError_t launch_toolbox<double>(const double *, ToolboxOut<double>, const Grid &, double, double *,
                                            int *, cudaStream_t);
template cudaError_t launch_band_maxabs<double>(const double *, const double *, double, const Grid &, double *,
                                                int *, cudaStream_t);

}  // namespace vsl
