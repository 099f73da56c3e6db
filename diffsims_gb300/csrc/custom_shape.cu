// Spot intensities from shape factors computed outside the kernels: the
// last step of SimulationGenerator.calculate_diffraction2d with a custom
// shape-factor function (diffsims/generators/simulation_generator.py:117-120,
// 387-411 calls any callable on each pattern's excitation errors).  A Python
// function cannot run in a kernel, so the orientation kernel selects the
// spots (the model switched off), the caller evaluates its function on their
// excitation errors, and this kernel finishes every pattern: I = sf |F|^2,
// the minimum-intensity mask I > max(I) * minimum_intensity (:237-240) and
// ordered compaction into a new CSR.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace ds {

constexpr int SHAPE_APPLY_THREADS = 256;

// One warp per pattern, patterns taken in order from a ticket; the output
// offset of a pattern comes from the decoupled look-back over patterns.
__global__ void __launch_bounds__(SHAPE_APPLY_THREADS)
apply_shape_kernel(const int64_t *__restrict__ off_in, const int32_t *__restrict__ idx_in,
                   const float4 *__restrict__ xyzi_in, const double *__restrict__ sf, const float *__restrict__ F2,
                   long long n, double thr, int64_t *__restrict__ off_out, int32_t *__restrict__ idx_out,
                   float4 *__restrict__ xyzi_out, long long capacity, int64_t *__restrict__ total, LookbackScratch lb,
                   int32_t *status) {
    const int lane = threadIdx.x & 31;
    const unsigned lanemask_lt = (1u << lane) - 1u;
    for (;;) {
        long long i = 0;
        if (lane == 0) i = (long long)atomicAdd(lb.ticket, 1ull);
        i = __shfl_sync(FULL_MASK, i, 0);
        if (i >= n) return;
        const long long a = off_in[i], b = off_in[i + 1];
        // I in the reference's order: shape factor times |F|^2 (FP64 product)
        auto inten = [&](long long k) -> double { return sf[k] * (double)F2[idx_in[k]]; };
        double mx = -INFINITY;
        for (long long k = a + lane; k < b; k += 32) mx = fmax(mx, inten(k));
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) mx = fmax(mx, __shfl_xor_sync(FULL_MASK, mx, d));
        const double cut = mx * thr;
        long long cnt = 0;
        for (long long k = a + lane; k < b; k += 32) cnt += inten(k) > cut ? 1 : 0;
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) cnt += __shfl_xor_sync(FULL_MASK, cnt, d);
        long long prefix = 0;
        if (lane == 0) {
            prefix = lookback_exclusive(lb, i, cnt, status);
            if (prefix >= 0) {
                off_out[i] = prefix;
                if (i == n - 1) {
                    off_out[n] = prefix + cnt;
                    *total = prefix + cnt;
                }
            }
        }
        prefix = __shfl_sync(FULL_MASK, prefix, 0);
        if (prefix < 0) return;  // a bounded wait gave up: DS_ERR_TIMEOUT is set
        long long pos = prefix;
        bool overflow = false;
        for (long long k0 = a; k0 < b; k0 += 32) {
            const long long k = k0 + lane;
            double I = 0.0;
            bool keep = false;
            if (k < b) {
                I = inten(k);
                keep = I > cut;
            }
            const unsigned bal = __ballot_sync(FULL_MASK, keep);
            if (keep) {
                const long long p = pos + __popc(bal & lanemask_lt);
                if (p < capacity) {
                    const float4 r = xyzi_in[k];
                    idx_out[p] = idx_in[k];
                    xyzi_out[p] = make_float4(r.x, r.y, r.z, (float)I);
                } else {
                    overflow = true;
                }
            }
            pos += __popc(bal);
        }
        if (__any_sync(FULL_MASK, overflow) && lane == 0) atomicOr(status, DS_ERR_CAPACITY);
    }
}

}  // namespace ds

using namespace ds;

extern "C" size_t ds_apply_shape_factors_scratch_bytes(int64_t n_patterns) {
    return n_patterns < 0 ? 0 : lookback_scratch_bytes(n_patterns);
}

extern "C" ds_status ds_apply_shape_factors(const int64_t *offsets_in, const int32_t *hkl_index_in,
                                            const float *xyzi_in, const double *shape_factors, const float *F2,
                                            int64_t n_patterns, double minimum_intensity, ds_spots *out,
                                            void *scratch, size_t scratch_bytes, int32_t *status, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_apply_shape_factors");
    DS_REQUIRE(out && status, "ds_apply_shape_factors: null pointer");
    DS_REQUIRE(n_patterns >= 0, "ds_apply_shape_factors: n_patterns < 0");
    DS_REQUIRE(std::isfinite(minimum_intensity), "ds_apply_shape_factors: minimum_intensity must be finite");
    DS_REQUIRE(out->hkl_index_bytes == 0 || out->hkl_index_bytes == 4,
               "ds_apply_shape_factors: hkl_index_bytes must be 0 or 4 (int32 rows)");
    cudaStream_t s = (cudaStream_t)stream;
    DS_REQUIRE(out->offsets && out->total, "ds_apply_shape_factors: null offsets / total");
    if (n_patterns == 0) {
        DS_CUDA_TRY(cudaMemsetAsync(out->offsets, 0, sizeof(int64_t), s));
        DS_CUDA_TRY(cudaMemsetAsync(out->total, 0, sizeof(int64_t), s));
        return DS_OK;
    }
    DS_REQUIRE(offsets_in, "ds_apply_shape_factors: null input offsets");
    DS_REQUIRE(out->capacity >= 0 && (out->capacity == 0 || (out->hkl_index && out->xyzi)),
               "ds_apply_shape_factors: output arrays missing");
    DS_REQUIRE(((uintptr_t)out->xyzi & 15) == 0 && ((uintptr_t)xyzi_in & 15) == 0,
               "ds_apply_shape_factors: xyzi arrays must be 16-byte aligned");
    DS_REQUIRE(scratch && scratch_bytes >= lookback_scratch_bytes(n_patterns),
               "ds_apply_shape_factors: scratch too small");
    DS_CUDA_TRY(cudaMemsetAsync(scratch, 0, lookback_scratch_bytes(n_patterns), s));
    int dev = 0, n_sm = 0, per_sm = 0;
    DS_CUDA_TRY(cudaGetDevice(&dev));
    DS_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    DS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, apply_shape_kernel, SHAPE_APPLY_THREADS, 0));
    // persistent: every warp resident, so a pattern's look-back only waits on
    // patterns whose warps are running
    const long long warps = (long long)n_sm * (per_sm > 0 ? per_sm : 1) * (SHAPE_APPLY_THREADS / 32);
    const long long blocks = (std::min(warps, (long long)n_patterns) + SHAPE_APPLY_THREADS / 32 - 1) /
                             (SHAPE_APPLY_THREADS / 32);
    apply_shape_kernel<<<(unsigned)blocks, SHAPE_APPLY_THREADS, 0, s>>>(
        offsets_in, hkl_index_in, reinterpret_cast<const float4 *>(xyzi_in), shape_factors, F2, n_patterns,
        minimum_intensity, out->offsets, out->hkl_index, reinterpret_cast<float4 *>(out->xyzi), out->capacity,
        out->total, lookback_scratch(scratch), status);
    return check_launch("apply_shape_kernel");
}
