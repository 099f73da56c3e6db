// A1 + A2: hkl box rule (host) and ordered hkl enumeration (device).
//
// Replaces ReciprocalLatticeVector.from_min_dspacing
// (diffsims/crystallography/reciprocal_lattice_vector.py:1131-1141): orix
// _get_highest_hkl (rule at diffsims/crystallography/get_hkl.py:49-57), the
// descending box without 000, the d >= d_min filter, the unique/ordered set
// and the trailing 000 rows.
#include <math.h>

#include <mutex>
#include <string>

#include "common.cuh"

namespace ds {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

// |g|^2 of integer hkl in the fixed operation order shared with the oracle:
// g = (h a* + k b*) + l c*, |g|^2 = (gx^2 + gy^2) + gz^2, round-to-nearest, no FMA.
__host__ __device__ inline double g2_fixed_order(const double *r, double h, double k, double l) {
#ifdef __CUDA_ARCH__
    double gx = __dadd_rn(__dadd_rn(__dmul_rn(h, r[0]), __dmul_rn(k, r[3])), __dmul_rn(l, r[6]));
    double gy = __dadd_rn(__dadd_rn(__dmul_rn(h, r[1]), __dmul_rn(k, r[4])), __dmul_rn(l, r[7]));
    double gz = __dadd_rn(__dadd_rn(__dmul_rn(h, r[2]), __dmul_rn(k, r[5])), __dmul_rn(l, r[8]));
    return __dadd_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gy, gy)), __dmul_rn(gz, gz));
#else
    volatile double gx = (h * r[0] + k * r[3]) + l * r[6];
    volatile double gy = (h * r[1] + k * r[4]) + l * r[7];
    volatile double gz = (h * r[2] + k * r[5]) + l * r[8];
    volatile double a = gx * gx;
    volatile double b = gy * gy;
    volatile double c = gz * gz;
    volatile double ab = a + b;
    return ab + c;
#endif
}

constexpr int ENUM_THREADS = 256;
constexpr int ENUM_ITEMS = 4;
constexpr int ENUM_TILE = ENUM_THREADS * ENUM_ITEMS;

// MODE 0: ReciprocalLatticeVector.from_min_dspacing -- descending box, 000
//         removed, keep 1/|g| >= dmin, n_zero trailing 000 rows.
// MODE 1: get_points_in_sphere (diffsims/utils/sim_utils.py:436-474) -- the
//         box in itertools.product order (h, then k, then l ascending from
//         -H, -K, -L), 000 kept in place, keep |g| < radius (held in dmin).
struct EnumConst {
    double r[9];
    double dmin;
    int32_t H, K, L;
    int32_t n_zero;
    long long total;    // box size
    long long n_tiles;
    long long capacity;
};

template <int MODE>
__global__ void __launch_bounds__(ENUM_THREADS)
enumerate_kernel(EnumConst c, int32_t *__restrict__ hkl_out, double *__restrict__ g2_out,
                 int64_t *__restrict__ count_out, LookbackScratch lb, int32_t *status) {
    __shared__ long long s_tile;
    __shared__ int s_warp[ENUM_THREADS / 32];
    __shared__ long long s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = (long long)atomicAdd(lb.ticket, 1ull);
    __syncthreads();
    const long long tile = s_tile;
    const int nl = 2 * c.L + 1, nk = 2 * c.K + 1;
    const long long base = tile * ENUM_TILE + (long long)tid * ENUM_ITEMS;

    int h[ENUM_ITEMS], k[ENUM_ITEMS], l[ENUM_ITEMS];
    double g2v[ENUM_ITEMS];
    bool keep[ENUM_ITEMS];
    int cnt = 0;
#pragma unroll
    for (int it = 0; it < ENUM_ITEMS; ++it) {
        long long i = base + it;
        keep[it] = false;
        if (i < c.total) {
            long long q = i / nl;
            if (MODE == 0) {
                l[it] = c.L - (int)(i - q * nl);
                k[it] = c.K - (int)(q % nk);
                h[it] = c.H - (int)(q / nk);
                if (h[it] != 0 || k[it] != 0 || l[it] != 0) {
                    double g2 = g2_fixed_order(c.r, (double)h[it], (double)k[it], (double)l[it]);
                    double d = __ddiv_rn(1.0, __dsqrt_rn(g2));
                    g2v[it] = g2;
                    keep[it] = d >= c.dmin;
                }
            } else {
                l[it] = (int)(i - q * nl) - c.L;
                k[it] = (int)(q % nk) - c.K;
                h[it] = (int)(q / nk) - c.H;
                double g2 = g2_fixed_order(c.r, (double)h[it], (double)k[it], (double)l[it]);
                g2v[it] = g2;
                keep[it] = __dsqrt_rn(g2) < c.dmin;
            }
        }
        cnt += keep[it] ? 1 : 0;
    }
    // block exclusive scan of per-thread counts
    int incl = warp_inclusive_scan(cnt, lane);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int v = lane < ENUM_THREADS / 32 ? s_warp[lane] : 0;
        int w = warp_inclusive_scan(v, lane);
        if (lane < ENUM_THREADS / 32) s_warp[lane] = w - v;  // exclusive warp offsets
        if (lane == ENUM_THREADS / 32 - 1) {
            long long prefix = lookback_exclusive(lb, tile, (long long)w, status);
            s_prefix = prefix;
            if (tile == c.n_tiles - 1 && prefix >= 0) {
                long long tot = prefix + w;
                for (int z = 0; z < c.n_zero; ++z) {
                    long long pos = tot + z;
                    if (pos < c.capacity) {
                        hkl_out[3 * pos] = 0; hkl_out[3 * pos + 1] = 0; hkl_out[3 * pos + 2] = 0;
                        g2_out[pos] = 0.0;
                    } else {
                        atomicOr(status, DS_ERR_CAPACITY);
                    }
                }
                *count_out = tot + c.n_zero;
            }
        }
    }
    __syncthreads();
    const long long prefix = s_prefix;
    if (prefix < 0) return;
    long long pos = prefix + s_warp[warp] + (incl - cnt);
#pragma unroll
    for (int it = 0; it < ENUM_ITEMS; ++it) {
        if (!keep[it]) continue;
        if (pos < c.capacity) {
            hkl_out[3 * pos] = h[it]; hkl_out[3 * pos + 1] = k[it]; hkl_out[3 * pos + 2] = l[it];
            g2_out[pos] = g2v[it];
        } else {
            atomicOr(status, DS_ERR_CAPACITY);
        }
        ++pos;
    }
}

}  // namespace ds

using namespace ds;

extern "C" ds_status ds_box_extent(const double recip[9], double min_dspacing, int32_t hmax_out[3]) {
    clear_error();
    DS_REQUIRE(recip && hmax_out, "ds_box_extent: null pointer");
    DS_REQUIRE(min_dspacing > 0 && isfinite(min_dspacing), "ds_box_extent: min_dspacing must be > 0");
    for (int i = 0; i < 3; ++i) {
        double e[3] = {0, 0, 0};
        double d = min_dspacing + 1;
        long long n = 0;
        while (d > min_dspacing) {
            ++n;
            DS_REQUIRE(n < (1 << 15), "ds_box_extent: box too large (lattice or radius out of range)");
            e[i] = (double)n;
            d = 1.0 / sqrt(g2_fixed_order(recip, e[0], e[1], e[2]));
            DS_REQUIRE(isfinite(d) || n == 1, "ds_box_extent: degenerate lattice");
        }
        hmax_out[i] = (int32_t)n;
    }
    return DS_OK;
}

extern "C" size_t ds_enumerate_scratch_bytes(const int32_t hmax[3]) {
    long long total = (long long)(2 * hmax[0] + 1) * (2 * hmax[1] + 1) * (2 * hmax[2] + 1);
    long long n_tiles = (total + ENUM_TILE - 1) / ENUM_TILE;
    return lookback_scratch_bytes(n_tiles);
}

extern "C" ds_status ds_enumerate_hkl(const double recip[9], const int32_t hmax[3], double min_dspacing,
                                      int32_t n_zero, int32_t *hkl_out, double *g2_out, int64_t capacity,
                                      int64_t *count_out, void *scratch, size_t scratch_bytes,
                                      int32_t *status, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_enumerate_hkl");
    DS_REQUIRE(recip && hmax && hkl_out && g2_out && count_out && scratch && status,
               "ds_enumerate_hkl: null pointer");
    DS_REQUIRE(hmax[0] >= 0 && hmax[1] >= 0 && hmax[2] >= 0, "ds_enumerate_hkl: negative box");
    DS_REQUIRE(n_zero >= 0 && n_zero <= 2, "ds_enumerate_hkl: n_zero must be 0, 1 or 2");
    DS_REQUIRE(min_dspacing > 0, "ds_enumerate_hkl: min_dspacing must be > 0");
    EnumConst c;
    for (int i = 0; i < 9; ++i) c.r[i] = recip[i];
    c.dmin = min_dspacing;
    c.H = hmax[0]; c.K = hmax[1]; c.L = hmax[2];
    c.n_zero = n_zero;
    c.total = (long long)(2 * c.H + 1) * (2 * c.K + 1) * (2 * c.L + 1);
    c.n_tiles = (c.total + ENUM_TILE - 1) / ENUM_TILE;
    c.capacity = capacity;
    DS_REQUIRE(capacity >= c.total + n_zero, "ds_enumerate_hkl: capacity below box size + n_zero");
    DS_REQUIRE(scratch_bytes >= lookback_scratch_bytes(c.n_tiles), "ds_enumerate_hkl: scratch too small");
    cudaStream_t s = (cudaStream_t)stream;
    DS_CUDA_TRY(cudaMemsetAsync(scratch, 0, lookback_scratch_bytes(c.n_tiles), s));
    enumerate_kernel<0><<<(unsigned)c.n_tiles, ENUM_THREADS, 0, s>>>(c, hkl_out, g2_out, count_out,
                                                                     lookback_scratch(scratch), status);
    return check_launch("enumerate_kernel");
}

extern "C" ds_status ds_enumerate_sphere(const double recip[9], const int32_t hmax[3], double radius,
                                         int32_t *hkl_out, double *g2_out, int64_t capacity, int64_t *count_out,
                                         void *scratch, size_t scratch_bytes, int32_t *status, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_enumerate_sphere");
    DS_REQUIRE(recip && hmax && hkl_out && g2_out && count_out && scratch && status,
               "ds_enumerate_sphere: null pointer");
    DS_REQUIRE(hmax[0] >= 0 && hmax[1] >= 0 && hmax[2] >= 0, "ds_enumerate_sphere: negative box");
    DS_REQUIRE(hmax[0] < (1 << 15) && hmax[1] < (1 << 15) && hmax[2] < (1 << 15), "ds_enumerate_sphere: box too large");
    DS_REQUIRE(radius > 0 && isfinite(radius), "ds_enumerate_sphere: radius must be > 0");
    EnumConst c;
    for (int i = 0; i < 9; ++i) c.r[i] = recip[i];
    c.dmin = radius;
    c.H = hmax[0]; c.K = hmax[1]; c.L = hmax[2];
    c.n_zero = 0;
    c.total = (long long)(2 * c.H + 1) * (2 * c.K + 1) * (2 * c.L + 1);
    c.n_tiles = (c.total + ENUM_TILE - 1) / ENUM_TILE;
    c.capacity = capacity;
    DS_REQUIRE(capacity >= c.total, "ds_enumerate_sphere: capacity below box size");
    DS_REQUIRE(scratch_bytes >= lookback_scratch_bytes(c.n_tiles), "ds_enumerate_sphere: scratch too small");
    cudaStream_t s = (cudaStream_t)stream;
    DS_CUDA_TRY(cudaMemsetAsync(scratch, 0, lookback_scratch_bytes(c.n_tiles), s));
    enumerate_kernel<1><<<(unsigned)c.n_tiles, ENUM_THREADS, 0, s>>>(c, hkl_out, g2_out, count_out,
                                                                     lookback_scratch(scratch), status);
    return check_launch("enumerate_kernel");
}

extern "C" const char *ds_last_error(void) { return ds::g_last_error.c_str(); }
extern "C" const char *ds_version(void) { return "diffsims_gb300 0.1.0 (sm_103a)"; }
