// mbarrier.cuh -- bounded waits on shared-memory mbarriers.
//
// No wait in this library spins without a limit: a wait that gives up returns
// false, the kernel sets ERR_TIMEOUT in its context's error word, lets its own
// asynchronous copies finish (again with a limit), and ends its work early;
// dr_context_check then reports DR_ERR_TIMEOUT.
#pragma once

#include <cstdint>

namespace dr {

// Polls of the production waits (the triangle-batch staging copies, the
// guiding kernels' weight copies and MMA commits).
constexpr uint32_t kMbarWaitPolls = 1u << 22;

// Polls mbarrier.try_wait.parity on the mbarrier at shared-memory address
// `bar` until the phase of parity `phase` has completed, at most `limit`
// times; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase, uint32_t limit)
{
    for (uint32_t it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

}  // namespace dr
