// async_copy.cuh -- bulk asynchronous copies into shared memory and the
// mbarriers that track them (sm_90+ PTX, used on sm_103a), with waits that
// give up after a time limit instead of spinning forever.
#pragma once
#include <cstdint>

namespace goofy_gpu {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes initialised barriers visible to the async (copy) proxy and the other threads' next reads.
__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// One arrival that also announces `bytes` of copies completing on the barrier.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// An L2 cache policy for data read once: its lines are the first L2 gives
// up when it needs room, so they do not push out lines still wanted (the
// rows the next launch prefetched, blocks not yet written back).
__device__ __forceinline__ uint64_t l2_evict_first_policy()
{
    uint64_t policy;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
    return policy;
}

// The same for half of the lines (the others keep the normal policy).
__device__ __forceinline__ uint64_t l2_evict_first_half_policy()
{
    uint64_t policy;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 0.5;" : "=l"(policy));
    return policy;
}

// Global memory -> shared memory, `bytes` (a multiple of 16, both addresses
// 16-byte aligned), completion counted on `bar`; the source lines get the L2
// cache policy `policy`.
__device__ __forceinline__ void bulk_copy_g2s_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                                   uint64_t policy)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

// Asks L2 to fetch `bytes` (a multiple of 16, 16-byte aligned address) of
// global memory.  A hint: nothing lands in the CTA, nothing completes on a
// barrier, and L2 stays coherent with every later write to those lines.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// A healthy pipeline waits microseconds; one second means a barrier that will
// never complete.
constexpr uint64_t kWaitLimitNs = 1000000000ull;

// Waits for the phase of `bar` with `parity` to complete.  Gives up (false)
// when `*abort` becomes non-zero or after kWaitLimitNs; a time-out raises
// *abort for the rest of the CTA and counts in *timeouts.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile uint32_t* abort,
                                          unsigned int* timeouts)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (abort && *abort) return false;
        if (global_ns() - t0 > kWaitLimitNs) {
            if (abort) *abort = 1u;
            atomicAdd(timeouts, 1u);
            return false;
        }
    }
}

}  // namespace goofy_gpu
