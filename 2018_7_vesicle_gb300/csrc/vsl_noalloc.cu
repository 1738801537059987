// vsl_noalloc.cu -- vsl_area_volume_noalloc_f64: the FP64 area/volume reduction for callers
// that cannot allocate device memory.
//
// Who cannot allocate: a caller that lives inside a host environment which owns the GPU's
// memory -- a MATLAB MEX function handed gpuArrays (MATLAB's memory manager owns and pools
// the device memory; memory taken around it is invisible to it and leaks when the MEX
// function errors out), or a framework whose caching allocator must not be bypassed -- and
// code in which the implicit device synchronisation of cudaMalloc/cudaFree is not allowed.
// Such a caller can pass F and the two output doubles but no workspace.
//
// The per-block partial sums of the reduction, which vsl_area_volume_f64 keeps in the
// caller's workspace, live here in one file-scope __device__ array of
// VSL_NOALLOC_SCRATCH_BYTES (1 MiB).  Every device that loads this library holds that
// array until the process exits.  Host code cannot use the array's name as a device
// address, so every call looks the address up (cudaGetSymbolAddress, a host-side query)
// on the device current at the call.  Nothing is cached: after a cudaDeviceReset the
// module is loaded again and the next call finds the new address.  The first call on a
// device is the one that loads the module there (lazy loading), so make it before any
// stream capture.  The entry point allocates nothing: no cudaMalloc, no cudaFree, no
// allocating library routine.
//
// The array is shared by every call on a device and keeps the last call's contents.
// Nothing in it needs to start at zero: the toolbox launch of a call writes every partial
// slot that the call's fixed-order sum reads.  Two calls whose launches can overlap on the
// GPU (unordered streams, or several host threads) race on the array.
#include <cmath>

#include "vsl_internal.h"

namespace vsl {
namespace {

static __device__ __align__(256) double noalloc_scratch[VSL_NOALLOC_SCRATCH_BYTES / sizeof(double)];

// device address of noalloc_scratch on the current device
int scratch_address(double **out)
{
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, noalloc_scratch) != cudaSuccess || p == nullptr) return VSL_ERR_CUDA;
    *out = static_cast<double *>(p);
    return VSL_OK;
}

}  // namespace
}  // namespace vsl

using namespace vsl;

extern "C" int vsl_area_volume_noalloc_f64(const double *F, double *area_volume, int rows, int cols, int pges,
                                           double dx, double dy, double dz, vsl_stream_t stream)
{
    if (F == nullptr || area_volume == nullptr) return VSL_ERR_NULL;
    if (int st = check_grid(rows, cols, pges, dx, dy, dz)) return st;
    const Grid g = make_grid(rows, cols, pges, dx, dy, dz);
    // two doubles (area, volume) per toolbox block
    const long long blocks = (long long)toolbox_partial_blocks(g);
    if (2 * blocks * (long long)sizeof(double) > (long long)VSL_NOALLOC_SCRATCH_BYTES) return VSL_ERR_SCRATCH_LIMIT;
    double *partials = nullptr;
    if (int st = scratch_address(&partials)) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const double ds = (dx + dy + dz) / 3;
    int nb = 0;
    if (launch_toolbox<double>(F, ToolboxOut<double>{}, g, ds, partials, &nb, s) != cudaSuccess) return VSL_ERR_CUDA;
    if (launch_sum_partials(partials, nb, 2, std::pow(ds, 3), area_volume, s) != cudaSuccess) return VSL_ERR_CUDA;
    return VSL_OK;
}
