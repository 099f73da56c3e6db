// Padded polar templates of spot patterns: Simulation2D.polar_flatten_simulations
// (diffsims/simulations/simulation2d.py:313-355) with
// DiffractingVector.to_flat_polar (diffsims/crystallography/_diffracting_vector.py:186-194)
// and get_closest (simulation2d.py:767-781), all patterns in one launch.
//
// One warp per pattern: r = |(x, y)| (x x + y y rounded as numpy does, no
// fused multiply-add), theta = atan2(y, x) in FP64 from the float32 spot
// positions; with axes, each value becomes the index of the closest axis
// entry (the upper one on ties, searchsorted from the left), spots whose
// indices reach the last entry of either axis are dropped, and the kept
// spots are compacted in order (ballot prefix).  Rows are padded with zeros
// to max_spots.  Reads 16 B and writes 24 B per spot slot: HBM-bound.
#include <algorithm>

#include "common.cuh"

namespace ds {

// numpy.searchsorted(a, v, side="left") then get_closest's correction
__device__ inline long long closest_index(const double *a, long long n, double v) {
    long long lo = 0, hi = n;  // first index with a[i] >= v
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    long long idx = lo;
    const long long prev = idx - 1 > 0 ? idx - 1 : 0;
    const long long here = idx < n - 1 ? idx : n - 1;
    if (idx == n || fabs(v - a[prev]) < fabs(v - a[here])) idx -= 1;
    return idx;
}

__global__ void polar_flatten_kernel(const int64_t *__restrict__ off, const float4 *__restrict__ xyzi,
                                     long long n_patterns, long long max_spots, const double *__restrict__ rax,
                                     long long n_r, const double *__restrict__ aax, long long n_a,
                                     double *__restrict__ r_out, double *__restrict__ t_out,
                                     double *__restrict__ i_out) {
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const bool binned = rax != nullptr && aax != nullptr;
    for (long long p = w0; p < n_patterns; p += nw) {
        const long long a = off[p], b = off[p + 1];
        const long long base = p * max_spots;
        long long kept = 0;
        for (long long j0 = a; j0 < b; j0 += 32) {
            const long long j = j0 + lane;
            bool keep = j < b;
            double rv = 0.0, tv = 0.0, iv = 0.0;
            if (keep) {
                const float4 e = xyzi[j];
                const double x = (double)e.x, y = (double)e.y;
                rv = sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
                tv = atan2(y, x);
                iv = (double)e.w;
                if (binned) {
                    const long long ir = closest_index(rax, n_r, rv), it = closest_index(aax, n_a, tv);
                    keep = ir < n_r - 1 && it < n_a - 1;
                    rv = (double)ir;
                    tv = (double)it;
                }
            }
            const unsigned bal = __ballot_sync(FULL_MASK, keep);
            if (keep) {
                const long long pos = base + kept + __popc(bal & ((1u << lane) - 1u));
                r_out[pos] = rv;
                t_out[pos] = tv;
                i_out[pos] = iv;
            }
            kept += __popc(bal);
        }
        for (long long k = kept + lane; k < max_spots; k += 32) {
            r_out[base + k] = 0.0;
            t_out[base + k] = 0.0;
            i_out[base + k] = 0.0;
        }
    }
}

}  // namespace ds

using namespace ds;

extern "C" ds_status ds_polar_flatten(const int64_t *offsets, const float *xyzi, int64_t n_patterns,
                                      int64_t max_spots, const double *radial_axes, int64_t n_radial,
                                      const double *azimuthal_axes, int64_t n_azimuthal, double *r_out,
                                      double *theta_out, double *intensity_out, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_polar_flatten");
    DS_REQUIRE(n_patterns >= 0 && max_spots >= 0, "ds_polar_flatten: negative size");
    DS_REQUIRE((radial_axes == nullptr) == (azimuthal_axes == nullptr),
               "ds_polar_flatten: give both axes or neither");
    DS_REQUIRE(radial_axes == nullptr || (n_radial > 0 && n_azimuthal > 0), "ds_polar_flatten: empty axes");
    if (n_patterns == 0 || max_spots == 0) return DS_OK;
    DS_REQUIRE(offsets && xyzi && r_out && theta_out && intensity_out, "ds_polar_flatten: null array");
    DS_REQUIRE(((uintptr_t)xyzi & 15) == 0, "ds_polar_flatten: xyzi must be 16-byte aligned");
    const long long warps = n_patterns;
    const long long blocks = std::min<long long>((warps * 32 + 255) / 256, 152LL * 16);
    polar_flatten_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
        offsets, reinterpret_cast<const float4 *>(xyzi), n_patterns, max_spots, radial_axes, n_radial,
        azimuthal_axes, n_azimuthal, r_out, theta_out, intensity_out);
    return check_launch("polar_flatten_kernel");
}
