// Bounded device-side waits on a counter that other blocks advance.
//
// Every spin in this library ends: after `limit` polls (with __nanosleep
// back-off) the wait reports failure, the caller records LH_FLAG_TIMEOUT in
// the frame's status word and leaves the stage, so a block that never
// arrives costs a flagged frame, never a hung GPU.
#pragma once

#include <cstdint>

#include "lh_internal.cuh"

namespace lh {

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// One thread waits until *counter >= target.  False when `limit` polls pass
// first, or when `flags` (the frame's status word; may be null) shows that
// another wait of the launch has already expired.
__device__ __forceinline__ bool counter_wait(const uint32_t* counter, uint32_t target, const uint32_t* flags,
                                             uint32_t limit) {
    uint32_t spins = 0;
    while (ld_acquire_u32(counter) < target) {
        if (++spins >= limit) return false;
        if (spins > 16) {
            if (flags && (*reinterpret_cast<const volatile uint32_t*>(flags) & LH_FLAG_TIMEOUT)) return false;
            __nanosleep(spins > 1024 ? 256 : 32);
        }
    }
    return true;
}

}  // namespace lh
