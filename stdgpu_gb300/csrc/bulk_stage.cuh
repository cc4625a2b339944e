// Staging of input tiles in shared memory with the TMA unit's bulk copies (cp.async.bulk, sm_90 and later),
// completed on shared-memory mbarriers.  Used by the bulk kernels to have a tile of input keys (or value_type
// pairs) in shared memory before the warps that probe it need it, so the probe of the home groups does not
// wait for the input load.  Single GPU, own memory only: no cluster multicast.
//
// Every wait is bounded: after kStageWaitNs of polling the waiter gives up, the caller records an error bit
// in the table header and stops issuing copies, and before the block exits it waits (bounded again) for
// the copies it has in flight.
#ifndef SG_BULK_STAGE_CUH
#define SG_BULK_STAGE_CUH

#include <cuda_runtime.h>

#include <cstdint>

#include "stdgpu_gb300/detail/layout.cuh"

namespace sg
{
namespace detail
{

constexpr unsigned int kErrStageWait = 4u;             // a bulk-copy wait gave up (table header error bit)
constexpr unsigned long long kStageWaitNs = 1000000000ull; // 1 s

SG_D uint32_t
smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

SG_D unsigned long long
global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

SG_D void
mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation and earlier shared-memory accesses of this thread visible to the bulk-copy
// (async) proxy.
SG_D void
fence_async_shared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One arrival that also announces `bytes` of bulk-copy data for the barrier's current phase.
SG_D void
mbar_arrive_expect(uint64_t* bar, uint32_t bytes)
{
    unsigned long long state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    (void)state;
}

// One plain arrival (completes a phase that expects no data).
SG_D void
mbar_arrive(uint64_t* bar)
{
    unsigned long long state;
    asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];" : "=l"(state) : "r"(smem_u32(bar)) : "memory");
    (void)state;
}

// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) from global to this block's
// shared memory; its completion counts against the barrier's expected bytes.
SG_D void
bulk_to_shared(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

SG_D bool
mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0u;
}

// Waits for the barrier phase with the given parity to complete; false after kStageWaitNs.
SG_D bool
mbar_wait(uint64_t* bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity))
    {
        return true;
    }
    const unsigned long long t0 = global_ns();
    while (true)
    {
        if (mbar_try_wait(bar, parity))
        {
            return true;
        }
        if (global_ns() - t0 > kStageWaitNs)
        {
            return false;
        }
    }
}

} // namespace detail
} // namespace sg

#endif
