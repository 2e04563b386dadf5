// tma.cuh -- tensor-memory-accelerator staging of the E box (inline PTX, sm_90+).
//
// The padded E field is described to the TMA unit as a 3-D tensor of reals
// {4*gx, gy, gz} (x fastest, 4 components per node interleaved), and a tile's
// box {4*sx, sy, sz} is fetched into the CTA's shared memory by one
// cp.async.bulk.tensor issued by one thread, completing on an mbarrier.
// Coordinates: x = 4*x0 (a multiple of 4 reals, so 16-byte aligned for both
// FP32 and FP64), y = y0, z = z0; the box never leaves the padded tensor.
// No cluster multicast is used.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace ohpic {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async (TMA) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_addr(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// Bounded wait for the barrier phase `parity`; false if it did not complete
// within max_iters polls (each poll may itself suspend briefly in hardware).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t max_iters)
{
    for (uint32_t it = 0; it < max_iters; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Polls allowed for the E box (tens of kilobytes from L2/HBM completes in
// microseconds; the bound only turns a lost completion into an error status).
constexpr uint32_t kTmaWaitPolls = 1u << 22;

}  // namespace ohpic
