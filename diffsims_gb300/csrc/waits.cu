// Bounded device waits: the process-wide wait limits and a probe whose waits
// nothing can satisfy (no counterpart in the reference, which has no device
// code on this path).
//
// Every spin in the library's kernels -- the decoupled look-back's wait for
// an earlier tile, the structure-factor kernels' wait for a TMA bulk copy --
// gives up after a number of polls, sets DS_ERR_TIMEOUT in the caller's
// status word and returns, so a lost wait never hangs the GPU.
// ds_set_wait_limits shortens (or restores) those limits for launches set up
// afterwards; ds_probe_wait_timeout runs both kinds of wait on flags that
// nothing ever sets, so a test can watch the limits work without faulting or
// hanging anything.
#include <atomic>

#include "common.cuh"

namespace ds {

static std::atomic<long long> g_lookback_limit{0};
static std::atomic<long long> g_mbarrier_limit{0};

long long wait_limit_lookback() {
    const long long v = g_lookback_limit.load(std::memory_order_relaxed);
    return v > 0 ? v : LB_SPIN_LIMIT;
}
long long wait_limit_mbarrier() {
    const long long v = g_mbarrier_limit.load(std::memory_order_relaxed);
    return v > 0 ? v : MBAR_SPIN_LIMIT;
}

// One block of 64 threads.  Thread 0 resolves tile 1 of a zeroed look-back
// (tile 0 never publishes); thread 32 waits on an mbarrier nobody arrives on
// and on which no copy was issued (so its drain wait may be short).
__global__ void wait_probe_kernel(LookbackScratch lb, long long polls, long long *out, int32_t *status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) out[0] = lookback_resolve(lb, 1, 5, status);
    if (threadIdx.x == 32) {
        mbar_init(&bar, 1);
        out[1] = mbar_wait_bounded(&bar, 0, status, polls, polls) ? 1 : 0;
    }
}

}  // namespace ds

using namespace ds;

extern "C" ds_status ds_set_wait_limits(int64_t lookback_polls, int64_t mbarrier_polls) {
    clear_error();
    g_lookback_limit.store(lookback_polls > 0 ? lookback_polls : 0, std::memory_order_relaxed);
    g_mbarrier_limit.store(mbarrier_polls > 0 ? mbarrier_polls : 0, std::memory_order_relaxed);
    return DS_OK;
}

extern "C" ds_status ds_probe_wait_timeout(int64_t polls, void *scratch, size_t scratch_bytes, int64_t *out,
                                           int32_t *status, void *stream) {
    clear_error();
    DS_REQUIRE(polls > 0 && polls <= (1ll << 20), "ds_probe_wait_timeout: polls must be in [1, 2^20]");
    DS_REQUIRE(scratch && out && status, "ds_probe_wait_timeout: null pointer");
    DS_REQUIRE(scratch_bytes >= lookback_scratch_bytes(2), "ds_probe_wait_timeout: scratch too small");
    cudaStream_t s = (cudaStream_t)stream;
    DS_CUDA_TRY(cudaMemsetAsync(scratch, 0, lookback_scratch_bytes(2), s));
    LookbackScratch lb = lookback_scratch(scratch);
    lb.spin_limit = polls;
    wait_probe_kernel<<<1, 64, 0, s>>>(lb, (long long)polls, reinterpret_cast<long long *>(out), status);
    return check_launch("wait_probe_kernel");
}
