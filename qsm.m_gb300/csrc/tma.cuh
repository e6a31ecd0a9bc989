// Tensor-memory-accelerator (TMA) loads and shared-memory mbarriers for
// sm_103a, as inline PTX: a tiled cp.async.bulk.tensor load of a 3-D box
// into shared memory that completes on an mbarrier, and the barrier
// operations around it (init, arrive with an expected byte count, bounded
// parity waits).  The tensor maps are built on the host (tma_encode_3d,
// common.cu) through the driver's cuTensorMapEncodeTiled, reached via the
// runtime's driver entry-point query so the library does not link libcuda.
//
// Rules kept by every caller: the box's innermost start coordinate times
// the element size is a multiple of 16 bytes (loads may start at negative or
// out-of-range coordinates and read zeros there); destinations are 128-byte
// aligned; loads never multicast; waits are bounded.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace qsm {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes initialised barriers visible to the async proxy (the TMA unit)
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_inval(uint64_t *bar)
{
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// one thread's arrival (its earlier shared-memory writes are released to the
// threads that then complete a wait on this phase)
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// the arrival of the issuing thread, announcing `bytes` of TMA traffic
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits until the barrier's phase with this parity has completed; false if
// it gave up after `limit` tries (each try suspends the thread for a
// hardware-defined time slice when the phase is not complete yet).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// One box of a 3-D tensor map into shared memory at dst; the transfer's
// bytes are counted on bar.  map is the address of a __grid_constant__
// kernel parameter.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace qsm
