// pf_async.cuh -- mbarrier + bulk asynchronous copy (TMA engine) helpers, inline PTX.
//
// cp.async.bulk copies a contiguous global range into shared memory and
// signals completion on an mbarrier with a transaction count.  Addresses must
// be 16-byte aligned and sizes multiples of 16 bytes; callers guarantee it.
// Every wait is bounded: mbar_wait returns false after 2 s of the global
// timer, so a kernel can raise its error flag and leave instead of hanging.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pf {

constexpr uint32_t kSpinLimit = 1u << 14;     // mbar_wait's default: the time bound below, not a poll count
constexpr uint32_t kSuspendHintNs = 100000;  // each poll may sleep this long unless the phase completes

static __device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

static __device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Arrive on `bar` (release: this thread's earlier shared-memory accesses
// are ordered before the phase completes).
static __device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Make initialised barriers visible to the asynchronous proxy.
static __device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's earlier generic-proxy shared-memory accesses before
// later asynchronous-proxy writes (a slot is refilled after it was read).
static __device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

static __device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// One poll; the thread sleeps until the phase completes or the hint elapses,
// so waiting warps do not take issue slots from working ones.
static __device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(kSuspendHintNs)
        : "memory");
    return ok != 0;
}

// Nanoseconds of the GPU's global timer.
static __device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr uint64_t kWaitNs = 2000000000ull;   // a wait gives up after 2 s of the global timer

// Bounded wait for phase `parity` of `bar` to complete: until kWaitNs has
// passed (the bound is time, not polls: a poll may return at once, so a
// count of polls can run out while a copy is merely slow), or, with an
// explicit `limit` (the failure-detection test), at most `limit` polls.
static __device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = kSpinLimit)
{
    if (limit != kSpinLimit) {
        for (uint32_t i = 0; i < limit; i++)
            if (mbar_try_wait(bar, parity)) return true;
        return false;
    }
    const uint64_t t0 = global_ns();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
}

// Global -> shared bulk copy of `bytes` (multiple of 16, both ends 16-byte
// aligned), completing `bytes` transactions on `bar`.
static __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Per-thread asynchronous 4-byte copy global -> shared (no alignment needs
// beyond the element's own).
static __device__ __forceinline__ void cp_async4(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

// Per-thread asynchronous 8-byte copy global -> shared (both addresses
// 8-byte aligned).
static __device__ __forceinline__ void cp_async8(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

// Per-thread asynchronous 16-byte copy global -> shared (both addresses
// 16-byte aligned), cached in L2 only.
static __device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

// Wait until this thread's earlier cp.async copies have landed.
static __device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// Arrive on `bar` once this thread's earlier cp.async copies have landed; the
// barrier's expected count must include one arrival per calling thread.
static __device__ __forceinline__ void cp_async_arrive(uint64_t* bar)
{
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

}  // namespace pf
