// vsl_tma.cuh -- tensor-memory-accelerator (TMA) plane loads for the 2.5D-tiled stage
// kernels: the PTX wrappers (mbarrier, cp.async.bulk.tensor) and the host encoding of a
// field's tensor map.
//
// A field is a 3-D tensor of FP32 (rows fastest, then columns, then pages); one copy brings
// a box of TMA_BOX_ROWS rows x TMA_BOX_COLS columns of one page into shared memory and
// completes on an mbarrier with its byte count.  The box's first row is a multiple of four
// (16 bytes), as the innermost coordinate of a tiled copy must be; rows outside the grid
// read as zero, so only tiles whose stencil halo lies inside the grid take this path.
#pragma once

#include <cuda.h>
#include <cstdint>

namespace vsl {

constexpr int TMA_BOX_ROWS = 40;  // 32 tile rows + 3 halo rows on each side, from a row 4 below
constexpr int TMA_BOX_COLS = 14;  // 8 tile columns + 3 halo columns on each side
constexpr unsigned TMA_PLANE_BYTES = TMA_BOX_ROWS * TMA_BOX_COLS * 4;
// a ring slot of the TMA layout: the box, padded to a multiple of 128 bytes (the alignment of
// a tensor copy's shared-memory destination)
constexpr int TMA_SLOT_FLOATS = 576;
static_assert(TMA_BOX_ROWS * TMA_BOX_COLS <= TMA_SLOT_FLOATS && (TMA_SLOT_FLOATS * 4) % 128 == 0, "slot layout");

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// make the barriers' initialisation visible to the async proxy (the copies complete on them)
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// this thread's arrival, announcing `bytes` of copies that complete on the barrier
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// one poll of the barrier's phase `parity`, suspending the thread for at most ~1 us
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(1000u)
        : "memory");
    return ok != 0u;
}

// order this thread's earlier generic-proxy shared-memory accesses before later copies
// (async proxy) into the same memory
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// one box of the tensor `tm` at (row x, column y, page z) into shared memory at dst
__device__ __forceinline__ void tma_load_box(void *dst, const CUtensorMap *tm, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(tm), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// Waits gave up: a copy did not complete within the bounded wait (the kernel goes on with
// the plane's earlier contents, every access still in bounds); read by vsl_tma_status.
__device__ unsigned tma_wait_timeouts;

// Waits for phase `parity` of the barrier, at most 2^16 polls of at most ~1 us each (a
// plane's copy completes within microseconds).  False when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    for (int it = 0; it < (1 << 16); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    atomicAdd(&tma_wait_timeouts, 1u);
    return false;
}

}  // namespace vsl
