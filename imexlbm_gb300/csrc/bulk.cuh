// Asynchronous bulk copies global -> shared memory (cp.async.bulk, the
// non-tensor TMA path) completed on an mbarrier, as inline PTX for sm_103a.
// Every wait is bounded: after a limit of SM clocks (WaitCtl::cycles,
// kWaitCycles unless a test lowers it) it reports failure and the caller
// records an error instead of spinning forever.
#pragma once

#include <cstdint>

namespace imex {

// Bounded-wait control handed to every kernel that waits on an mbarrier:
// where a wait that ran out is recorded (bit 0 of *err), the wait limit in
// SM clocks, and a test hook - CTA `starve_cta` (-1: none) arms the first
// stage of its ring without issuing that stage's copies, so its first wait
// runs out with no copy in flight.  make_wait_ctl (lattice.cu) fills it
// from the process's test-fault setting (imex_test_set_fault).
struct WaitCtl {
    unsigned* err;
    long long cycles;
    int starve_cta;
};
WaitCtl make_wait_ctl(unsigned* err);

namespace bulk {

constexpr long long kWaitCycles = 1ll << 31;  // ~1 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make mbarrier initialisation visible to the async proxy.
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's earlier generic-proxy shared-memory accesses (made
// visible to it by a CTA barrier) before its next async-proxy writes.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bytes from global src to shared dst (both 16-byte aligned, bytes a
// multiple of 16), completing `bytes` transactions on bar.
__device__ __forceinline__ void copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
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

// Wait for phase `parity` of bar to complete; false after `cycles` SM clocks.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long cycles)
{
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > cycles) return false;
    return true;
}

}  // namespace bulk
}  // namespace imex
