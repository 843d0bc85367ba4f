// les_tma.cuh -- Tensor Memory Accelerator (TMA) copies and mbarriers for the
// marching stencil kernels (sm_100-family PTX: cp.async.bulk.tensor,
// mbarrier.*).  Every wait is bounded.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdint.h>

namespace les {

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that also announces `bytes` of expected transaction count.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for phase `parity` of the barrier.  Gives up after ~2^22 polls
// (each try_wait may suspend for a bounded time) and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity)
{
    for (unsigned it = 0; it < (1u << 22); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// After a wait on the plane `cur` gave up: waits again (bounded) on every
// ring slot whose copy was issued -- planes cur .. min(cur + ahead, last) --
// so that a late copy lands before the CTA leaves and its shared memory is
// handed to another CTA.  `phase` bit s is the parity the next wait on slot
// s expects.  If these bounded waits also give up, the copy never completes
// and the CTA leaves anyway: an unbounded wait there would hang the GPU.  The
// TMA-staged passes are off by default (LES_OPT_TMA).
__device__ __forceinline__ void mbar_drain(uint64_t* bar, unsigned phase, int ring, int cur, int ahead, int last)
{
    for (int q = 0; q <= ahead && cur + q <= last; ++q) {
        const int s = (cur + q) % ring;
        mbar_wait_bounded(&bar[s], (phase >> s) & 1u);
    }
}

// 3-D tiled TMA load of the box at element coordinates (x, y, z) into shared
// memory; completion is signalled on `bar` as transaction bytes.  x times
// the element size must be a multiple of 16 bytes; coordinates outside the
// tensor read as zero.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// Host: encode a 3-D tiled tensor map over a dense [nx][ny][nz] array
// (innermost k), box {bx, by, 1}.  Returns false when the driver entry point
// is unavailable or the encoding is rejected.
bool tma_encode_3d(CUtensorMap* map, CUtensorMapDataType dtype, size_t esize, void* base, int nx, int ny, int nz,
                   unsigned bx, unsigned by);

}  // namespace les
