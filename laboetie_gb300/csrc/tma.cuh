// tma.cuh -- bulk tensor copies (TMA, cp.async.bulk.tensor) into shared memory completed on
// shared-memory mbarriers (sm_90+): barrier init, arrive with an expected byte count, a
// time-bounded parity wait, and a 4-D tiled load.  A tensor map is passed by the generic
// address of a __grid_constant__ kernel parameter.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace lbg {

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

// one arrival per phase; the bulk copies complete the transaction bytes
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes the initialised barriers visible to the asynchronous (bulk copy) proxy
__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(
                     smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase of the given parity to complete: at most about limit_ns of global time
// (2 s by default, and 2^28 polls should the timer not advance); false if it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity,
                                          unsigned long long limit_ns = 2000000000ull)
{
    const unsigned s = smem_addr(bar);
    unsigned long long t0 = 0;
    for (unsigned it = 0; it < (1u << 28); ++it) {
        unsigned ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(ok)
                     : "r"(s), "r"(parity)
                     : "memory");
        if (ok) return true;
        if ((it & 63u) == 0u) {
            const unsigned long long t = global_ns();
            if (it == 0u) t0 = t;
            else if (t - t0 > limit_ns) return false;
        }
    }
    return false;
}

// Tiled 4-D load of the tensor map's box at coordinates (c0, c1, c2, c3) (innermost first) into
// shared memory at dst (128-byte aligned), completing its bytes on bar.
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            int c3, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace lbg
