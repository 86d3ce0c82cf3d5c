// Diagnostic launches that run each kind of bounded device-side wait of the
// library -- the decoupled look-back of the culls, the grid barrier of the
// persistent frame kernel, the mbarrier wait of the TMA-staged resolve --
// against a condition that is either met at once or never met (a
// predecessor that never publishes, a block that never arrives, an
// mbarrier arrival that never comes), with a caller-chosen poll limit.  The
// expired case must come back as LH_FLAG_TIMEOUT in a status word the host
// reads, with the launch finished and the context usable: that is the whole
// failure-handling contract of the frame kernels.  No counterpart in the
// reference (Vulkan has no user-visible device waits).
#include "cull_phases.cuh"
#include "tma.cuh"
#include "waits.cuh"

namespace lh {
namespace {

// words: [0, 1] look-back status words of tiles 0 and 1, [2] barrier counter
// (low 32 bits), [3] status word (low 32 bits: LH_FLAG_*), [4] the wait's
// result (the look-back's exclusive prefix, or 1 when the wait completed).
__global__ void k_check_wait(uint32_t which, uint32_t limit, uint32_t satisfied, unsigned long long* words) {
    __shared__ uint64_t bar;
    uint32_t* flags = reinterpret_cast<uint32_t*>(words + 3);
    if (which == LH_WAIT_LOOKBACK) {
        // tile 1 looks back (the whole warp) at tile 0, which publishes 5 or never
        if (satisfied && threadIdx.x == 0) st_status(reinterpret_cast<uint64_t*>(&words[0]), kStatIncl | 5u);
        __syncwarp();
        const uint64_t excl = lookback_warp(reinterpret_cast<uint64_t*>(words), 1, 7, flags, limit);
        if (threadIdx.x == 0) words[4] = excl;
    } else if (which == LH_WAIT_GRID_BARRIER) {
        if (threadIdx.x == 0) {
            // this block arrives; a second block that never launches would be needed
            uint32_t* counter = reinterpret_cast<uint32_t*>(words + 2);
            atomicAdd(counter, 1u);
            const bool ok = counter_wait(counter, satisfied ? 1u : 2u, flags, limit);
            if (!ok) atomicOr(flags, LH_FLAG_TIMEOUT);
            words[4] = ok ? 1u : 0u;
        }
    } else {
        if (threadIdx.x == 0) {
            // expected arrivals: 1 (met by the one below) or 2 (never met)
            mbar_init(&bar, satisfied ? 1u : 2u);
            mbar_arrive(&bar);
            const bool ok = mbar_wait(&bar, 0u, limit);
            if (!ok) atomicOr(flags, LH_FLAG_TIMEOUT);
            words[4] = ok ? 1u : 0u;
        }
    }
}

}  // namespace
}  // namespace lh

extern "C" lh_status lh_check_bounded_wait(uint32_t which, uint32_t poll_limit, uint32_t satisfied,
                                           uint64_t* d_words, void* stream) {
    using namespace lh;
    if (which > LH_WAIT_MBARRIER || poll_limit == 0 || poll_limit > kSpinLimit || !d_words ||
        ((uintptr_t)d_words & 7))
        return LH_ERR_INVALID_ARGUMENT;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(d_words, 0, 8 * sizeof(uint64_t), s) != cudaSuccess) return LH_ERR_CUDA;
    k_check_wait<<<1, 32, 0, s>>>(which, poll_limit, satisfied ? 1u : 0u,
                                  reinterpret_cast<unsigned long long*>(d_words));
    return cudaGetLastError() == cudaSuccess ? LH_OK : LH_ERR_CUDA;
}
