// Bulk asynchronous copies (TMA, cp.async.bulk) and mbarrier helpers, in inline PTX for sm_90+
// (used here on sm_103a).
#pragma once

#include <cstdint>

namespace lbmg {

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes the initialised barrier visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arrive once and announce `bytes` of incoming transactions on the barrier.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// L2 policy for the streamed populations. Evict first keeps the small per-cell arrays (flags,
// link entries, handler records) in L2 between steps; it is used when every cell is updated by a
// row block. Edge blocks re-read rows that row blocks have just streamed, so domains with edge
// cells keep the normal policy.
__device__ __forceinline__ uint64_t l2_stream_policy(bool evict_first)
{
    uint64_t pol;
    if (evict_first)
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    else
        asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// Global -> shared bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned),
// completing on `bar`, with L2 cache policy `pol`.
__device__ __forceinline__ void bulk_g2s_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar, uint64_t pol)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}

// One poll of phase `parity` of `bar`. The thread may sleep up to kWaitHintNs inside it while the
// phase is incomplete (it wakes as soon as the phase completes), so that a waiting warp issues a
// handful of polls instead of spinning.
constexpr uint32_t kWaitHintNs = 2000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kWaitHintNs)
        : "memory");
    return ok != 0;
}

// Waits for phase `parity` of `bar` with a bounded number of polls (at most about
// max_polls * kWaitHintNs). Returns false (and the caller reports an error) if the phase did not
// complete in time.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_polls)
{
    for (uint32_t k = 0; k < max_polls; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Asynchronous 16-byte copy global -> shared (both 16-byte aligned), and the wait for all of the
// calling thread's such copies.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem_dst)), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// A hint: the L1 line at p is fetched now, for a read that follows later.
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// Programmatic dependent launch (griddepcontrol). grid_dep_wait blocks until the kernel this grid
// follows in its stream has completed and its writes are visible; it returns at once for a launch
// without the programmatic attribute. grid_dep_launch lets the next kernel in the stream, if it was
// launched with that attribute, start its blocks once every block of this grid has issued it or
// exited; they then wait in their own grid_dep_wait.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

}  // namespace lbmg
