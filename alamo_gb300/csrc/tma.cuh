// tma.cuh -- inline-PTX helpers shared by the sm_103a kernels that move data
// with the Tensor Memory Accelerator and complete it on shared-memory
// mbarriers: barrier set-up, transaction-count arming, bounded waits, and the
// tensor (tiled) and bulk (linear) copies into shared memory.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace agb {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// One arrival (release semantics at CTA scope) on a barrier initialised with
// the number of arriving threads.
__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Bounded wait for the phase of parity `parity` to complete: false after
// about 2^31 clock cycles (~1 s at 2 GHz) without completion.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    const long long t0 = clock64();
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > (1LL << 31)) return false;
    }
}

// 4-D tiled tensor copy global -> shared, completing on `bar`.  The innermost
// coordinate x times the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load4(uint32_t dst, const CUtensorMap* map, int x, int y, int z, int c,
                                          uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(c), "r"(bar)
        : "memory");
}

// Linear bulk copy global -> shared of `bytes` (a multiple of 16; both
// addresses 16-byte aligned), completing on `bar`.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
                 : "memory");
}

}  // namespace agb
