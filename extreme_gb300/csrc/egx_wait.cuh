// Bounded waits on shared-memory mbarriers, shared by every kernel that waits
// for a TMA copy: a wait polls mbarrier.try_wait.parity against %globaltimer
// and gives up after limit_ns, so that a copy that never lands becomes an
// error status (EGX_ERR_TIMEOUT in the context's device flag, read by the
// host after the launch) instead of a hung GPU.
#pragma once

#include <cstdint>

namespace egx {

__device__ __forceinline__ uint64_t wait_clock_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// true when the phase of parity `parity` of the barrier at shared address
// `bar` has completed
__device__ __forceinline__ bool mbar_try_parity(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// true when the phase completed within limit_ns, false when the wait gave up
__device__ __forceinline__ bool mbar_wait_ns(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
    const uint64_t t0 = wait_clock_ns();
    while (!mbar_try_parity(bar, parity))
        if (wait_clock_ns() - t0 > limit_ns) return false;
    return true;
}

}  // namespace egx
