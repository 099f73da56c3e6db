// Shared device/host helpers of the diffsims_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>

#include <nvtx3/nvToolsExt.h>

#include "diffsims_gb300.h"

namespace ds {

// An NVTX range over the host work of one C entry (argument checks, plans,
// the enqueued launches), named after the entry: profilers (Nsight Systems,
// ncu's NVTX filters) show each call on the host timeline beside its
// kernels.  Without a profiler attached a push / pop is a check of a null
// callback.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
#define DS_NVTX_RANGE(name) ::ds::NvtxRange ds_nvtx_range_(name)

// ----------------------------------------------------------------------------
// host-side error reporting (thread-local last message)
// ----------------------------------------------------------------------------
void set_error(const std::string &msg);
void clear_error();

#define DS_REQUIRE(cond, msg)                                   \
    do {                                                        \
        if (!(cond)) {                                          \
            ::ds::set_error(msg);                               \
            return DS_ERR_INVALID_ARGUMENT;                     \
        }                                                       \
    } while (0)

#define DS_CUDA_TRY(expr)                                                          \
    do {                                                                           \
        cudaError_t _e = (expr);                                                   \
        if (_e != cudaSuccess) {                                                   \
            ::ds::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));   \
            return DS_ERR_CUDA;                                                    \
        }                                                                          \
    } while (0)

// Bounds-checked builds (-DDS_DEBUG_BOUNDS; the library is then built as
// libdiffsims_gb300_debug.so): DS_IN_BOUNDS(i, n, status) is false, and
// DS_ERR_BOUNDS is or-ed into the kernel's status word, when the index i lies
// outside [0, n); the caller skips the access.  Normal builds compile every
// check to `true`.
#ifdef DS_DEBUG_BOUNDS
__device__ __forceinline__ bool debug_in_bounds(long long i, long long n, int32_t *status) {
    if (i >= 0 && i < n) return true;
    atomicOr(status, DS_ERR_BOUNDS);
    return false;
}
#define DS_IN_BOUNDS(i, n, status) ::ds::debug_in_bounds((long long)(i), (long long)(n), (status))
#else
#define DS_IN_BOUNDS(i, n, status) true
#endif

inline ds_status check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string(what) + ": " + cudaGetErrorString(e));
        return DS_ERR_CUDA;
    }
    return DS_OK;
}

constexpr unsigned FULL_MASK = 0xffffffffu;

// ----------------------------------------------------------------------------
// double-float ("dd") arithmetic on FP32 pairs: Dekker / Knuth error-free
// transformations (Dekker, Numer. Math. 18 (1971) 224; Knuth TAOCP vol. 2,
// 4.2.2).  The explicit _rn intrinsics keep the compiler from contracting or
// reassociating the compensation terms.
// ----------------------------------------------------------------------------
struct dd {
    float hi, lo;
};

__device__ __forceinline__ dd two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ dd quick_two_sum(float a, float b) {  // |a| >= |b|
    float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dd two_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    float t = __fadd_rn(__fadd_rn(a.lo, b.lo), s.lo);
    return quick_two_sum(s.hi, t);
}
__device__ __forceinline__ dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
__device__ __forceinline__ dd dd_add_f(dd a, float b) {
    dd s = two_sum(a.hi, b);
    return quick_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ dd dd_mul(dd a, dd b) {
    dd p = two_prod(a.hi, b.hi);
    float t = __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi));
    return quick_two_sum(p.hi, __fadd_rn(p.lo, t));
}
__device__ __forceinline__ dd dd_mul_f(dd a, float b) {
    dd p = two_prod(a.hi, b);
    return quick_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
__device__ __forceinline__ dd dd_abs(dd a) { return a.hi < 0.f ? dd_neg(a) : a; }

__host__ __device__ inline void split_double(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

// ----------------------------------------------------------------------------
// decoupled look-back: ordered exclusive prefix of per-tile counts in one pass
// (Merrill & Garland, "Single-pass Parallel Prefix Scan with Decoupled
// Look-back", NVIDIA TR 2016).  Tile state word: bits 62..63 = flag
// (0 empty, 1 aggregate, 2 inclusive prefix), bits 0..61 = value.
// Tiles take tickets in launch order (atomicAdd), so a tile only ever waits on
// tiles that already run; every wait is bounded and reports DS_ERR_TIMEOUT.
// ----------------------------------------------------------------------------
constexpr unsigned long long LB_FLAG_AGG = 1ull << 62;
constexpr unsigned long long LB_FLAG_INC = 2ull << 62;
constexpr unsigned long long LB_VALUE_MASK = (1ull << 62) - 1;
constexpr long long LB_SPIN_LIMIT = 1ll << 24;  // polls (with backoff) before giving up (default)

// Process-wide wait limits read when a launch is set up (ds_set_wait_limits;
// 0 = the defaults above and below).
long long wait_limit_lookback();
long long wait_limit_mbarrier();

struct LookbackScratch {
    unsigned long long *ticket;  // one word, zeroed before launch
    unsigned long long *state;   // n_tiles words, zeroed before launch
    long long spin_limit;        // polls before a wait gives up
};

inline size_t lookback_scratch_bytes(long long n_tiles) {
    return (size_t)(n_tiles + 32) * sizeof(unsigned long long);
}
inline LookbackScratch lookback_scratch(void *base) {
    auto *p = reinterpret_cast<unsigned long long *>(base);
    return {p, p + 32, wait_limit_lookback()};
}

// A state word carries its flag and value together and no other data is
// handed over through it, so relaxed gpu-scope accesses suffice.  (A release
// store would wait for every write the CTA issued before the barrier that
// precedes it -- a whole tile's staging -- before publishing.)
__device__ __forceinline__ unsigned long long lb_load(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void lb_store(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Publish a tile's count (its inclusive prefix directly for tile 0).  ONE thread.
__device__ inline void lookback_publish(LookbackScratch lb, long long tile, long long count) {
    lb_store(lb.state + tile, (tile == 0 ? LB_FLAG_INC : LB_FLAG_AGG) | ((unsigned long long)count & LB_VALUE_MASK));
}

// Exclusive prefix of a tile whose count was published; publishes its
// inclusive prefix.  ONE thread.  On timeout returns -1 and sets
// DS_ERR_TIMEOUT in *status.
__device__ inline long long lookback_resolve(LookbackScratch lb, long long tile, long long count, int32_t *status) {
    if (tile == 0) return 0;
    long long excl = 0;
    long long idx = tile - 1;
    long long spins = 0;
    unsigned ns = 8;
    while (true) {
        unsigned long long s = lb_load(lb.state + idx);
        unsigned long long flag = s & ~LB_VALUE_MASK;
        if (flag == 0ull) {
            if (++spins > lb.spin_limit) {
                atomicOr(status, DS_ERR_TIMEOUT);
                return -1;
            }
            __nanosleep(ns);
            if (ns < 256) ns <<= 1;
            continue;
        }
        excl += (long long)(s & LB_VALUE_MASK);
        if (flag == LB_FLAG_INC) break;
        --idx;
    }
    lb_store(lb.state + tile, LB_FLAG_INC | ((unsigned long long)(excl + count) & LB_VALUE_MASK));
    return excl;
}

// Publish and resolve in one go.  ONE thread.
__device__ inline long long lookback_exclusive(LookbackScratch lb, long long tile, long long count,
                                               int32_t *status) {
    lookback_publish(lb, tile, count);
    return lookback_resolve(lb, tile, count, status);
}

// ----------------------------------------------------------------------------
// 1-D bulk copies global -> shared through the TMA unit (cp.async.bulk) with an
// mbarrier transaction count.  Addresses 16-byte aligned, sizes multiples of 16.
// ----------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
constexpr long long MBAR_SPIN_LIMIT = 1ll << 22;  // default polls of the first wait
// Bounded wait for phase `parity` (`limit` polls); on timeout flags
// DS_ERR_TIMEOUT and waits a second bounded time (`drain` polls; by default
// the long fixed one, whatever `limit` is) so that no copy this CTA issued is
// left writing its shared memory after it returns.  A caller that issued no
// copy on the barrier may pass a short `drain`.  Returns false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int32_t *status,
                                                  long long limit = MBAR_SPIN_LIMIT,
                                                  long long drain = 16 * MBAR_SPIN_LIMIT) {
    for (long long i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(status, DS_ERR_TIMEOUT);
    for (long long i = 0; i < drain; ++i)
        if (mbar_try_wait(bar, parity)) break;
    return false;
}

__device__ __forceinline__ int warp_inclusive_scan(int v, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int n = __shfl_up_sync(FULL_MASK, v, d);
        if (lane >= d) v += n;
    }
    return v;
}

__device__ __forceinline__ long long warp_exclusive_scan_ll(long long v, int lane) {
    long long incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const long long n = __shfl_up_sync(FULL_MASK, incl, d);
        if (lane >= d) incl += n;
    }
    return incl - v;
}

}  // namespace ds
