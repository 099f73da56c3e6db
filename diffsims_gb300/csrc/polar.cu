// Padded polar templates of spot patterns: Simulation2D.polar_flatten_simulations
// (diffsims/simulations/simulation2d.py:313-355) with
// DiffractingVector.to_flat_polar (diffsims/crystallography/_diffracting_vector.py:186-194)
// and get_closest (simulation2d.py:767-781), all patterns in one launch.
//
// r = |(x, y)| (x x + y y rounded as numpy does, no fused multiply-add),
// theta = atan2(y, x) in FP64 from the float32 spot positions; with axes,
// each value becomes the index of the closest axis entry (the upper one on
// ties, searchsorted from the left), spots whose indices reach the last entry
// of either axis are dropped, and the kept spots are compacted in order
// (ballot prefix, one warp per pattern).  Rows are padded with zeros to
// max_spots.  Reads 16 B and writes 24 B per spot slot.  On GB300 the FP64
// atan2 and square root bound the kernels (FP64 issues at 1/64 of the FP32
// rate).  The FP32 variant (ds_polar_flatten_f32) computes r and theta with
// sqrtf / atan2f and searches float copies of the axes: within ~2e-7 of the
// FP64 values, the error the float32 spot positions already carry, and bound
// by the bytes instead.
#include <algorithm>
#include <type_traits>

#include "common.cuh"

namespace ds {

// numpy.searchsorted(a, v, side="left") then get_closest's correction.  The
// search starts from the position a uniform axis would give (inv = (n - 1) /
// (a[n-1] - a[0]), 0 when degenerate): two compares settle it for the
// linspace axes templates use; a bisection of what remains finishes any other
// sorted axis.  The answer (the first i with !(a[i] < v), n if none) is the
// bisection's for every input: each step keeps it inside [lo, hi].
template <typename T>
__device__ inline long long closest_index(const T *a, long long n, T v, T inv) {
    long long lo = 0, hi = n;
    const T gf = (v - a[0]) * inv;
    long long g = 0;
    if (gf > (T)0) g = gf < (T)(n - 1) ? (long long)gf : n - 1;  // NaN: 0
    if (a[g] < v) lo = g + 1;
    else hi = g;
    if (lo == g + 1) {
        if (lo < hi) {
            if (a[lo] < v) lo = lo + 1;
            else hi = lo;
        }
    } else if (lo < hi) {
        if (a[hi - 1] < v) lo = hi;
        else hi = hi - 1;
    }
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

template <typename T>
__device__ inline T uniform_inverse(const T *a, long long n) {
    return (n > 1 && a[n - 1] > a[0]) ? (T)(n - 1) / (a[n - 1] - a[0]) : (T)0;
}

// float -> double and small unsigned -> double by assembling the IEEE bits
// with integer instructions only: both conversions are exact, and on this GPU
// the conversion instructions issue on the scarce FP64 pipe (a predicated-off
// fallback would still issue, so every case is integer arithmetic).
__device__ __forceinline__ double f2d_bits(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    unsigned long long E, M;
    if (e == 0xffu) {  // infinities and NaNs (the quiet bit lands on the double's)
        E = 0x7ffull;
        M = (unsigned long long)m << 29;
    } else if (e != 0u) {  // normal: rebias 127 -> 1023
        E = e + 896u;
        M = (unsigned long long)m << 29;
    } else if (m != 0u) {  // subnormal: m 2^-149 = 1.x 2^(k-149), k the top bit of m
        const int k = 31 - __clz(m);
        E = (unsigned long long)(k + 874);
        M = ((unsigned long long)m << (52 - k)) & ((1ull << 52) - 1ull);
    } else {  // signed zero
        E = 0ull;
        M = 0ull;
    }
    return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) | (E << 52) | M));
}
__device__ __forceinline__ double u2d_bits(unsigned n) {
    if (n == 0u) return 0.0;
    const int e = 31 - __clz(n);  // n = 1.m * 2^e
    const unsigned long long m = ((unsigned long long)n << (52 - e)) & ((1ull << 52) - 1ull);
    return __longlong_as_double((long long)(((unsigned long long)(e + 1023) << 52) | m));
}

// r, theta (FP32 or FP64) and the intensity of one spot record
template <bool F32>
__device__ __forceinline__ void polar_values(const float4 &e, double &rv, double &tv, double &iv, float &rf,
                                             float &tf) {
    if constexpr (F32) {
        rf = sqrtf(__fadd_rn(__fmul_rn(e.x, e.x), __fmul_rn(e.y, e.y)));
        tf = atan2f(e.y, e.x);
        rv = f2d_bits(rf);
        tv = f2d_bits(tf);
    } else {
        const double x = f2d_bits(e.x), y = f2d_bits(e.y);
        rv = sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
        tv = atan2(y, x);
    }
    iv = f2d_bits(e.w);
}

// Unbinned templates keep every spot in place (slot k of pattern p holds its
// spot k), so each slot is independent: one short block per pattern (many
// resident at once hide each other's latency), its threads over the slots
// (spots, then the zero padding), four slices' loads issued before any is
// used.
constexpr int POLAR_FLAT_THREADS = 128, POLAR_FLAT_UNROLL = 4;
template <bool F32>
__global__ void __launch_bounds__(POLAR_FLAT_THREADS)
polar_flat_kernel(const int64_t *__restrict__ off, const float4 *__restrict__ xyzi, long long n_patterns,
                  long long max_spots, double *__restrict__ r_out, double *__restrict__ t_out,
                  double *__restrict__ i_out) {
    for (long long p = blockIdx.x; p < n_patterns; p += gridDim.x) {
        const long long a = off[p], cnt = off[p + 1] - a;
        const long long base = p * max_spots;
        for (long long k0 = threadIdx.x; k0 < max_spots; k0 += POLAR_FLAT_UNROLL * POLAR_FLAT_THREADS) {
            float4 e[POLAR_FLAT_UNROLL];
#pragma unroll
            for (int u = 0; u < POLAR_FLAT_UNROLL; ++u) {
                const long long k = k0 + u * POLAR_FLAT_THREADS;
                e[u] = k < cnt ? xyzi[a + k] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < POLAR_FLAT_UNROLL; ++u) {
                const long long k = k0 + u * POLAR_FLAT_THREADS;
                if (k < max_spots) {
                    double rv = 0.0, tv = 0.0, iv = 0.0;
                    if (k < cnt) {
                        float rf, tf;
                        polar_values<F32>(e[u], rv, tv, iv, rf, tf);
                    }
                    r_out[base + k] = rv;
                    t_out[base + k] = tv;
                    i_out[base + k] = iv;
                }
            }
        }
    }
}

// Binned templates: the closest-axis indices, spots at the last entry of
// either axis dropped and the rest compacted in order.  One warp per
// pattern, two slices of 32 spots per step (both loads issued before either
// is used).
template <bool F32>
__global__ void polar_binned_kernel(const int64_t *__restrict__ off, const float4 *__restrict__ xyzi,
                                    long long n_patterns, long long max_spots,
                                    const std::conditional_t<F32, float, double> *__restrict__ rax, long long n_r,
                                    const std::conditional_t<F32, float, double> *__restrict__ aax, long long n_a,
                                    double *__restrict__ r_out, double *__restrict__ t_out,
                                    double *__restrict__ i_out) {
    using AX = std::conditional_t<F32, float, double>;
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const AX inv_r = uniform_inverse(rax, n_r), inv_a = uniform_inverse(aax, n_a);
    for (long long p = w0; p < n_patterns; p += nw) {
        const long long a = off[p], b = off[p + 1];
        const long long base = p * max_spots;
        long long kept = 0;
        // one slice: indices, then the kept spots compacted in order
        auto emit = [&](const float4 &e, bool keep) {
            double rv = 0.0, tv = 0.0, iv = 0.0;
            if (keep) {
                float rf, tf;
                polar_values<F32>(e, rv, tv, iv, rf, tf);
                long long ir, it;
                if constexpr (F32) {
                    ir = closest_index<float>(rax, n_r, rf, inv_r);
                    it = closest_index<float>(aax, n_a, tf, inv_a);
                } else {
                    ir = closest_index<double>(rax, n_r, rv, inv_r);
                    it = closest_index<double>(aax, n_a, tv, inv_a);
                }
                // 0 <= index < n - 1 for every kept spot: exact small integers
                keep = ir < n_r - 1 && it < n_a - 1;
                rv = u2d_bits((unsigned)ir);
                tv = u2d_bits((unsigned)it);
            }
            const unsigned bal = __ballot_sync(FULL_MASK, keep);
            if (keep) {
                const long long pos = base + kept + __popc(bal & ((1u << lane) - 1u));
                r_out[pos] = rv;
                t_out[pos] = tv;
                i_out[pos] = iv;
            }
            kept += __popc(bal);
        };
        for (long long j0 = a; j0 < b; j0 += 64) {
            const long long j = j0 + lane, j2 = j + 32;
            const bool k1 = j < b, k2 = j2 < b;
            float4 e1 = make_float4(0.f, 0.f, 0.f, 0.f), e2 = e1;
            if (k1) e1 = xyzi[j];
            if (k2) e2 = xyzi[j2];
            emit(e1, k1);
            if (j0 + 32 < b) emit(e2, k2);  // warp-uniform
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

template <bool F32, typename AX>
static ds_status polar_flatten(const char *name, const int64_t *offsets, const float *xyzi, int64_t n_patterns,
                               int64_t max_spots, const AX *radial_axes, int64_t n_radial, const AX *azimuthal_axes,
                               int64_t n_azimuthal, double *r_out, double *theta_out, double *intensity_out,
                               void *stream) {
    const std::string w(name);
    DS_REQUIRE(n_patterns >= 0 && max_spots >= 0, w + ": negative size");
    DS_REQUIRE((radial_axes == nullptr) == (azimuthal_axes == nullptr), w + ": give both axes or neither");
    DS_REQUIRE(radial_axes == nullptr || (n_radial > 0 && n_azimuthal > 0), w + ": empty axes");
    if (n_patterns == 0 || max_spots == 0) return DS_OK;
    DS_REQUIRE(offsets && xyzi && r_out && theta_out && intensity_out, w + ": null array");
    DS_REQUIRE(((uintptr_t)xyzi & 15) == 0, w + ": xyzi must be 16-byte aligned");
    const cudaStream_t st = (cudaStream_t)stream;
    if (radial_axes == nullptr) {
        const long long blocks = std::min<long long>(n_patterns, 0x7fffffffLL);
        polar_flat_kernel<F32><<<(unsigned)blocks, POLAR_FLAT_THREADS, 0, st>>>(
            offsets, reinterpret_cast<const float4 *>(xyzi), n_patterns, max_spots, r_out, theta_out, intensity_out);
        return check_launch("polar_flat_kernel");
    }
    const long long blocks = std::min<long long>((n_patterns * 32 + 255) / 256, 152LL * 16);
    polar_binned_kernel<F32><<<(unsigned)blocks, 256, 0, st>>>(
        offsets, reinterpret_cast<const float4 *>(xyzi), n_patterns, max_spots, radial_axes, n_radial,
        azimuthal_axes, n_azimuthal, r_out, theta_out, intensity_out);
    return check_launch("polar_binned_kernel");
}

extern "C" ds_status ds_polar_flatten(const int64_t *offsets, const float *xyzi, int64_t n_patterns,
                                      int64_t max_spots, const double *radial_axes, int64_t n_radial,
                                      const double *azimuthal_axes, int64_t n_azimuthal, double *r_out,
                                      double *theta_out, double *intensity_out, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_polar_flatten");
    return polar_flatten<false>("ds_polar_flatten", offsets, xyzi, n_patterns, max_spots, radial_axes, n_radial,
                                azimuthal_axes, n_azimuthal, r_out, theta_out, intensity_out, stream);
}

extern "C" ds_status ds_polar_flatten_f32(const int64_t *offsets, const float *xyzi, int64_t n_patterns,
                                          int64_t max_spots, const float *radial_axes, int64_t n_radial,
                                          const float *azimuthal_axes, int64_t n_azimuthal, double *r_out,
                                          double *theta_out, double *intensity_out, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_polar_flatten_f32");
    return polar_flatten<true>("ds_polar_flatten_f32", offsets, xyzi, n_patterns, max_spots, radial_axes,
                               n_radial, azimuthal_axes, n_azimuthal, r_out, theta_out, intensity_out, stream);
}
