// Detector images of spot patterns (the reference's per-pattern
// Simulation2D.get_diffraction_pattern, diffsims/simulations/simulation2d.py:357-442,
// with diffsims/pattern/detector_functions.py:251-359), many patterns per launch.
//
// Per pattern, in one CTA of a persistent grid:
//   1. every spot -> pixel coordinates in FP64 (divide by the calibration,
//      in-plane rotation / mirror, shift to the direct beam), the in-frame test;
//   2. fast mode: truncate to whole pixels and keep, per pixel, the LAST spot
//      (numpy's assignment order) through a shared-memory hash of pixel ->
//      largest spot index; sub-pixel mode: each spot's clip box;
//   3. ordered compaction of the surviving spots with their row / column ranges;
//   4. the image row by row, one warp per row: the spots covering the row
//      (ballot over the compacted list), each adding amp * rowweight *
//      colweight into the lanes' column registers, stored as float4 streams.
// Fast mode is a delta image filtered by scipy.ndimage.gaussian_filter (mode
// "reflect", radius int(truncate sigma + 0.5), weights exp(-x^2 / 2 sigma^2)
// normalised); the filter is separable and linear, so every spot adds
// I * A(y, Y) * A(x, X) with A the 1-D weight including the mirrored images of
// the half-sample symmetric extension.  Sub-pixel mode adds
// I / (2 pi sigma^2) exp(-d^2 / 2 sigma^2) over the spot's box.  Rows no spot
// reaches are written as zeros directly; normalisation takes a first pass over
// the covered rows for the maximum.
//
// The image is the only large traffic (4 H W bytes per pattern, written once):
// the kernel is bound by HBM writes.
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "common.cuh"

namespace ds {

constexpr int RAS_THREADS = 256;
constexpr int RAS_WARPS = RAS_THREADS / 32;
constexpr int RAS_K = 2;                  // float4 column chunks per lane in one row segment
constexpr int RAS_SEG = 32 * 4 * RAS_K;   // columns per row segment
constexpr int RAS_MAX_R = 511;            // fast mode: largest filter radius
constexpr size_t RAS_SMEM_LIMIT = 200 * 1024;

struct RasterConst {
    int H, W, R;
    int fast, normalize;
    int one_pass;       // fast + normalise: build each covered row once (flags below)
    int NS, T;          // arena capacity in spots, hash slots (power of two >= 2 NS)
    double cal, cx, cy, ca, sa, mf, snap;
    float icf, caf, saf, mff, cxf, cyf, snapf;  // FP32 copies (1 / cal rounded) for the cell pre-check
    double pref, exp_pref, clip;
    float wt[RAS_MAX_R + 1];  // fast: filter weights w[|d|], d = 0..R
};

struct RasterArena {
    int *key;     // fast: pixel index Y W + X, or -1; sub-pixel: 0 kept / -1
    int *slot;    // fast: hash slot of the spot
    int *hkey, *hidx;
    float *amp;
    int *ylo, *yhi, *xlo, *xhi;
    double *px, *py;
    unsigned *rows;  // covered-row bitmap
    int *misc;       // warp totals (RAS_WARPS), scalars
    float *wmax;     // per-warp maxima (RAS_WARPS)
};

__host__ __device__ inline size_t ras_align(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t raster_arena_bytes(int NS, int T, int H) {
    size_t o = 0;
    o += ras_align((size_t)NS * 4) * 2;       // key, slot
    o += ras_align((size_t)T * 4) * 2;        // hkey, hidx
    o += ras_align((size_t)NS * 4) * 5;       // amp, ylo, yhi, xlo, xhi
    o += ras_align((size_t)NS * 8) * 2;       // px, py
    o += ras_align((size_t)((H + 31) / 32) * 4);
    o += ras_align(64 * 4) + ras_align(RAS_WARPS * 4);
    return o;
}

__device__ inline RasterArena carve(unsigned char *base, int NS, int T, int H) {
    RasterArena A;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + o;
        o += ras_align(bytes);
        return p;
    };
    A.key = (int *)take((size_t)NS * 4);
    A.slot = (int *)take((size_t)NS * 4);
    A.hkey = (int *)take((size_t)T * 4);
    A.hidx = (int *)take((size_t)T * 4);
    A.amp = (float *)take((size_t)NS * 4);
    A.ylo = (int *)take((size_t)NS * 4);
    A.yhi = (int *)take((size_t)NS * 4);
    A.xlo = (int *)take((size_t)NS * 4);
    A.xhi = (int *)take((size_t)NS * 4);
    A.px = (double *)take((size_t)NS * 8);
    A.py = (double *)take((size_t)NS * 8);
    A.rows = (unsigned *)take((size_t)((H + 31) / 32) * 4);
    A.misc = (int *)take(64 * 4);
    A.wmax = (float *)take(RAS_WARPS * 4);
    return A;
}

// Pixel coordinates of one spot, in the reference's order of operations:
// divide by the calibration, rotate by the in-plane angle (mirrored: negated
// azimuth), shift to the direct beam.  For angle 0 the rotation is exact.
__device__ inline void pixel_xy(const RasterConst &c, float4 e, double &X, double &Y) {
    const double u = (double)e.x / c.cal, v = c.mf * ((double)e.y / c.cal);
    X = (u * c.ca - v * c.sa) + c.cx;
    Y = (v * c.ca + u * c.sa) + c.cy;
    if (c.snap > 0.0) {
        const double rx = rint(X), ry = rint(Y);
        if (fabs(X - rx) <= c.snap) X = rx;
        if (fabs(Y - ry) <= c.snap) Y = ry;
    }
}

__device__ inline bool in_frame(const RasterConst &c, double X, double Y) {
    return X >= 0.0 && X < (double)c.W && Y >= 0.0 && Y < (double)c.H;
}

// Whole-pixel cell (ix, iy) of one spot and the frame test, as pixel_xy and
// in_frame give them in FP64 (fast mode needs nothing else).  The same
// arithmetic in FP32 is within E = 4 * 2^-23 (|u| + |v| + |c| + |X|) + 1e-6 px
// of the FP64 X (the rounding of 1 / cal, u, v, cos, sin and the two FMAs,
// with a factor of two to spare); when both FP32 coordinates lie farther than
// E plus the snap window from every pixel edge, their floors are the FP64
// floors (and no snapping applies), else the FP64 path decides.  Non-finite
// or huge coordinates fail the test and take the FP64 path.
__device__ inline bool pixel_cell(const RasterConst &c, float4 e, int &ix, int &iy) {
    const float u = e.x * c.icf, v = c.mff * (e.y * c.icf);
    const float Xf = fmaf(u, c.caf, fmaf(-v, c.saf, c.cxf));
    const float Yf = fmaf(v, c.caf, fmaf(u, c.saf, c.cyf));
    const float ex = 4.77e-7f * (fabsf(u) + fabsf(v) + fabsf(c.cxf) + fabsf(Xf)) + 1e-6f + c.snapf;
    const float ey = 4.77e-7f * (fabsf(u) + fabsf(v) + fabsf(c.cyf) + fabsf(Yf)) + 1e-6f + c.snapf;
    const float fx = Xf - floorf(Xf), fy = Yf - floorf(Yf);
    if (fx > ex && fx < 1.f - ex && fy > ey && fy < 1.f - ey) {
        ix = (int)floorf(Xf);
        iy = (int)floorf(Yf);
        return ix >= 0 && ix < c.W && iy >= 0 && iy < c.H;
    }
    double X, Y;
    pixel_xy(c, e, X, Y);
    if (!in_frame(c, X, Y)) return false;
    ix = (int)X;
    iy = (int)Y;
    return true;
}

// Sub-pixel mode: the clip radius of a spot (NaN: the spot is skipped),
// detector_functions.py:337-343.
__device__ inline double clip_radius(const RasterConst &c, double I) {
    return sqrt(log(c.clip / (c.pref * I)) / c.exp_pref);
}

// 1-D filter weight that a delta at P contributes to position x on a line of
// n pixels: sum over d in [-R, R] of w[|d|] where the half-sample symmetric
// extension (period 2n) maps x + d onto P.
__device__ inline float reflect_weight(const RasterConst &c, int x, int P, int n) {
    const int R = c.R;
    float v = 0.f;
    if (R < n) {
        const int d = abs(x - P);
        if (d <= R) v += c.wt[d];
        const int m1 = x + P + 1;          // image at -P-1
        if (m1 <= R) v += c.wt[m1];
        const int m2 = 2 * n - 1 - P - x;  // image at 2n-1-P
        if (m2 <= R) v += c.wt[m2];
        return v;
    }
    // images P + 2kn and 2kn - 1 - P within [x - R, x + R]
    const int per = 2 * n;
    for (int fam = 0; fam < 2; ++fam) {
        const int base = fam == 0 ? P : -P - 1;
        const int k0 = (int)floor((double)(x - R - base) / per);
        for (int k = k0;; ++k) {
            const int q = base + k * per;
            if (q > x + R) break;
            if (q >= x - R) v += c.wt[abs(q - x)];
        }
    }
    return v;
}

__device__ __forceinline__ float row_weight(const RasterConst &c, const RasterArena &A, int k, int y) {
    if (c.fast) return reflect_weight(c, y, (int)A.py[k], c.H);
    const double dy = (double)y - A.py[k];
    return expf((float)(c.exp_pref * dy * dy));
}

__device__ __forceinline__ float col_weight(const RasterConst &c, const RasterArena &A, int k, int x) {
    if (c.fast) return reflect_weight(c, x, (int)A.px[k], c.W);
    const double dx = (double)x - A.px[k];
    return expf((float)(c.exp_pref * dx * dx));
}

__device__ __forceinline__ void st_cs(float4 *p, float4 v) {
    asm volatile("st.global.cs.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}
__device__ __forceinline__ void st_cs1(float *p, float v) {
    asm volatile("st.global.cs.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

// One row segment [x0, x0 + RAS_SEG) of row y: lane registers acc[i][e] for
// columns x0 + (lane + 32 i) * 4 + e.
__device__ inline void row_segment(const RasterConst &c, const RasterArena &A, int n_alive, int y, int x0,
                                   int lane, float (&acc)[RAS_K][4]) {
#pragma unroll
    for (int i = 0; i < RAS_K; ++i)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[i][e] = 0.f;
    const int x1 = x0 + RAS_SEG;
    for (int k0 = 0; k0 < n_alive; k0 += 32) {
        const int k = k0 + lane;
        bool cov = false;
        float a = 0.f;
        if (k < n_alive) {
            cov = A.ylo[k] <= y && y < A.yhi[k] && A.xlo[k] < x1 && A.xhi[k] > x0;
            if (cov) a = A.amp[k] * row_weight(c, A, k, y);
        }
        unsigned m = __ballot_sync(FULL_MASK, cov);
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            const float ab = __shfl_sync(FULL_MASK, a, b);
            const int kk = k0 + b;
            const int xl = A.xlo[kk], xh = A.xhi[kk];
#pragma unroll
            for (int i = 0; i < RAS_K; ++i) {
                const int base = x0 + (lane + 32 * i) * 4;
                if (base < xh && base + 4 > xl) {
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int x = base + e;
                        if (x >= xl && x < xh) acc[i][e] = fmaf(ab, col_weight(c, A, kk, x), acc[i][e]);
                    }
                }
            }
        }
    }
}

template <bool VEC>
__global__ void __launch_bounds__(RAS_THREADS, 4) raster_kernel(const RasterConst c, const int64_t *__restrict__ off,
                                                             const float4 *__restrict__ xyzi, long long n_patterns,
                                                             float *__restrict__ out, unsigned char *gscratch,
                                                             size_t arena_bytes, int32_t *status) {
    extern __shared__ __align__(16) unsigned char ras_smem[];
    unsigned char *base = gscratch ? gscratch + (size_t)blockIdx.x * arena_bytes : ras_smem;
    const RasterArena A = carve(base, c.NS, c.T, c.H);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int H = c.H, W = c.W;
    const size_t img = (size_t)H * W;
    const int nwords = (H + 31) / 32;

    for (long long p = blockIdx.x; p < n_patterns; p += gridDim.x) {
        const long long a0 = off[p];
        const long long n_ll = off[p + 1] - a0;
        if (n_ll > c.NS || n_ll < 0) {
            if (tid == 0) atomicOr(status, DS_ERR_CAPACITY);
            continue;
        }
        const int n = (int)n_ll;
        int Tp = 64;
        while (Tp < 2 * n) Tp <<= 1;
        const int tbits = __ffs(Tp) - 1;
        if (c.fast) {
            for (int t = tid; t < Tp; t += RAS_THREADS) {
                A.hkey[t] = -1;
                A.hidx[t] = -1;
            }
        }
        if (tid == 0) A.misc[RAS_WARPS] = 0;  // in-frame count
        __syncthreads();

        // ---- 1-2: pixel coordinates, frame test, last-write-wins per pixel
        int my_in = 0;
        for (int i = tid; i < n; i += RAS_THREADS) {
            const float4 e = xyzi[a0 + i];
            double X, Y;
            pixel_xy(c, e, X, Y);
            int key = -1;
            if (in_frame(c, X, Y)) {
                ++my_in;
                if (c.fast) {
                    key = (int)Y * W + (int)X;
                    // open addressing; Tp >= 2 n slots, so a free slot is always found
                    unsigned h = ((unsigned)key * 2654435761u) >> (32 - tbits);
                    int sl = -1;
                    for (int t = 0; t < Tp; ++t) {
                        const int prev = atomicCAS(&A.hkey[h], -1, key);
                        if (prev == -1 || prev == key) {
                            atomicMax(&A.hidx[h], i);
                            sl = (int)h;
                            break;
                        }
                        h = (h + 1) & (unsigned)(Tp - 1);
                    }
                    A.slot[i] = sl;
                    if (sl < 0) key = -1;
                } else {
                    const double rad = clip_radius(c, (double)e.w);
                    if (!isnan(rad)) key = 0;
                }
            }
            A.key[i] = key;
        }
        my_in = __reduce_add_sync(FULL_MASK, my_in);
        if (lane == 0 && my_in) atomicAdd(&A.misc[RAS_WARPS], my_in);
        __syncthreads();
        const int n_in = A.misc[RAS_WARPS];

        // ---- 3: ordered compaction of the surviving spots
        int n_alive = 0;
        for (int c0 = 0; c0 < n; c0 += RAS_THREADS) {
            const int i = c0 + tid;
            bool alive = false;
            if (i < n && A.key[i] >= 0) alive = !c.fast || A.hidx[A.slot[i]] == i;  // slot >= 0 when key >= 0
            const unsigned bal = __ballot_sync(FULL_MASK, alive);
            if (lane == 0) A.misc[warp] = __popc(bal);
            __syncthreads();
            int wbase = 0, tot = 0;
            for (int w = 0; w < RAS_WARPS; ++w) {
                const int v = A.misc[w];
                if (w < warp) wbase += v;
                tot += v;
            }
            if (alive) {
                const int k = n_alive + wbase + __popc(bal & ((1u << lane) - 1));
                const float4 e = xyzi[a0 + i];
                if (c.fast) {
                    const int key = A.key[i];
                    const int X = key % W, Y = key / W;
                    A.px[k] = (double)X;
                    A.py[k] = (double)Y;
                    A.amp[k] = e.w;
                    A.ylo[k] = max(0, Y - c.R);
                    A.yhi[k] = min(H, Y + c.R + 1);
                    A.xlo[k] = max(0, X - c.R);
                    A.xhi[k] = min(W, X + c.R + 1);
                } else {
                    double X, Y;
                    pixel_xy(c, e, X, Y);
                    const double rad = clip_radius(c, (double)e.w);
                    A.px[k] = X;
                    A.py[k] = Y;
                    A.amp[k] = (float)((double)e.w * c.pref);
                    A.ylo[k] = (int)fmax(0.0, ceil(Y - rad));
                    A.yhi[k] = (int)fmin((double)H, floor(Y + rad + 1.0));
                    A.xlo[k] = (int)fmax(0.0, ceil(X - rad));
                    A.xhi[k] = (int)fmin((double)W, floor(X + rad + 1.0));
                }
            }
            n_alive += tot;
            __syncthreads();
        }

        // ---- covered rows
        for (int w = tid; w < nwords; w += RAS_THREADS) A.rows[w] = 0u;
        __syncthreads();
        for (int k = tid; k < n_alive; k += RAS_THREADS) {
            const int lo = A.ylo[k], hi = A.yhi[k];
            for (int y = lo; y < hi;) {
                const int wi = y >> 5, b0 = y & 31;
                const int nb = min(32 - b0, hi - y);
                const unsigned m = (nb == 32 ? 0xffffffffu : ((1u << nb) - 1u)) << b0;
                atomicOr(&A.rows[wi], m);
                y += nb;
            }
        }
        __syncthreads();

        // ---- maximum over the image (normalise)
        float mx = 1.f;
        const bool norm = c.normalize && n_in > 0;
        if (norm) {
            float wm = -INFINITY;
            bool any_empty_row = false;
            for (int y = warp; y < H; y += RAS_WARPS) {
                if (!((A.rows[y >> 5] >> (y & 31)) & 1u)) {
                    any_empty_row = true;
                    continue;
                }
                for (int x0 = 0; x0 < W; x0 += RAS_SEG) {
                    float acc[RAS_K][4];
                    row_segment(c, A, n_alive, y, x0, lane, acc);
#pragma unroll
                    for (int i = 0; i < RAS_K; ++i)
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (x0 + (lane + 32 * i) * 4 + e < W) wm = fmaxf(wm, acc[i][e]);
                }
            }
            if (any_empty_row) wm = fmaxf(wm, 0.f);
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) wm = fmaxf(wm, __shfl_xor_sync(FULL_MASK, wm, d));
            if (lane == 0) A.wmax[warp] = wm;
            __syncthreads();
            mx = A.wmax[0];
            for (int w = 1; w < RAS_WARPS; ++w) mx = fmaxf(mx, A.wmax[w]);
        }

        // ---- the image
        float *dst = out + (size_t)p * img;
        const float zero_val = norm ? 0.f / mx : 0.f;
        for (int y = warp; y < H; y += RAS_WARPS) {
            float *row = dst + (size_t)y * W;
            const bool covered = (A.rows[y >> 5] >> (y & 31)) & 1u;
            if (!covered) {
                if (VEC) {
                    const float4 z = make_float4(zero_val, zero_val, zero_val, zero_val);
                    for (int x = lane * 4; x < W; x += 128) st_cs(reinterpret_cast<float4 *>(row + x), z);
                } else {
                    for (int x = lane; x < W; x += 32) st_cs1(row + x, zero_val);
                }
                continue;
            }
            for (int x0 = 0; x0 < W; x0 += RAS_SEG) {
                float acc[RAS_K][4];
                row_segment(c, A, n_alive, y, x0, lane, acc);
#pragma unroll
                for (int i = 0; i < RAS_K; ++i) {
                    const int xb = x0 + (lane + 32 * i) * 4;
                    float v[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) v[e] = norm ? acc[i][e] / mx : acc[i][e];
                    if (VEC) {
                        if (xb < W) st_cs(reinterpret_cast<float4 *>(row + xb), make_float4(v[0], v[1], v[2], v[3]));
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (xb + e < W) st_cs1(row + xb + e, v[e]);
                    }
                }
            }
        }
        __syncthreads();  // the arena is reused by the next pattern
    }
}

// ------------------------------------------------------------ fast mode ----
// Whole-pixel spots and the Gaussian filter (simulation2d.py:425-431 with
// detector_functions.py:287-294).  Every surviving spot's footprint is at
// most P = 2R + 1 rows by P columns, with separable weights precomputed per
// spot (the 1-D reflect-mode weights, rw and cw).  Per-row spot lists (CSR,
// each row's spots in ascending spot order, so sums are deterministic) let one
// warp build a row in a shared-memory row buffer: per listed spot, P lanes add
// amp * rw * cw to their columns.
struct FastArena {
    int *key, *slot, *hkey, *hidx;
    float *amp;
    int *sx, *sy;       // whole-pixel spot position
    float *cw;          // NS x P column weights
    int2 *ent;          // row entries: (amp * row weight as bits, X << 16 | spot)
    int *rcnt, *rstart, *rfill;  // H + 1 each
    float *rowbuf;      // RAS_WARPS x RAS_FSEG
    unsigned *flags;    // one pass: per (row, segment, half) the lanes whose float4 is non-zero
    int *misc;
    float *wmax;
};
constexpr int RAS_FSEG = 256;  // columns per row segment (32 lanes x 2 float4)
constexpr size_t RAS_FLAGS_MAX = 32 * 1024;  // bytes of one-pass flags the arena may hold
__host__ __device__ inline size_t fast_flag_bytes(int H, int W) { return (size_t)H * ((W + RAS_FSEG - 1) / RAS_FSEG) * 8; }

__host__ __device__ inline size_t fast_arena_bytes(int NS, int T, int H, int P, size_t flag_bytes) {
    size_t o = 0;
    o += ras_align((size_t)NS * 4) * 2;              // key, slot
    o += ras_align((size_t)T * 4) * 2;               // hkey, hidx
    o += ras_align((size_t)NS * 4) * 3;              // amp, sx, sy
    o += ras_align((size_t)NS * P * 4);              // cw
    o += ras_align((size_t)NS * P * 8);              // ent
    o += ras_align((size_t)(H + 1) * 4) * 3;         // rcnt, rstart, rfill
    o += ras_align((size_t)RAS_WARPS * RAS_FSEG * 4);
    o += ras_align(flag_bytes);
    o += ras_align(64 * 4) + ras_align(RAS_WARPS * 4);
    return o;
}

__device__ inline FastArena carve_fast(unsigned char *base, int NS, int T, int H, int P, size_t flag_bytes) {
    FastArena A;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + o;
        o += ras_align(bytes);
        return p;
    };
    A.key = (int *)take((size_t)NS * 4);
    A.slot = (int *)take((size_t)NS * 4);
    A.hkey = (int *)take((size_t)T * 4);
    A.hidx = (int *)take((size_t)T * 4);
    A.amp = (float *)take((size_t)NS * 4);
    A.sx = (int *)take((size_t)NS * 4);
    A.sy = (int *)take((size_t)NS * 4);
    A.cw = (float *)take((size_t)NS * P * 4);
    A.ent = (int2 *)take((size_t)NS * P * 8);
    A.rcnt = (int *)take((size_t)(H + 1) * 4);
    A.rstart = (int *)take((size_t)(H + 1) * 4);
    A.rfill = (int *)take((size_t)(H + 1) * 4);
    A.rowbuf = (float *)take((size_t)RAS_WARPS * RAS_FSEG * 4);
    A.flags = (unsigned *)take(flag_bytes);
    A.misc = (int *)take(64 * 4);
    A.wmax = (float *)take(RAS_WARPS * 4);
    return A;
}

__device__ __forceinline__ void st_wb(float4 *p, float4 v) { *p = v; }  // default policy: stays in L2 for the rescale

// Row y, columns [x0, x0 + RAS_FSEG) into the warp's buffer; on return lane l
// holds columns x0 + 4 l + (0..3) in v[0..3] and x0 + 128 + 4 l + (0..3) in v[4..7].
// An entry carries amp * (row weight) and the spot's column X; its columns
// are [max(0, X - R), min(W, X + R + 1)) with weights cw[spot][x - max(0, X - R)].
__device__ inline void fast_row_segment(const RasterConst &c, const FastArena &A, int P, int y, int x0, int lane,
                                        float *buf, float (&v)[8]) {
    float4 *b4 = reinterpret_cast<float4 *>(buf);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    b4[lane] = z;
    b4[lane + 32] = z;
    __syncwarp();
    const int e0 = A.rstart[y], e1 = A.rstart[y + 1];
    for (int e = e0; e < e1; ++e) {
        const int2 en = A.ent[e];
        const int X = en.y >> 16, k = en.y & 0xffff;
        const int xl = max(0, X - c.R), xh = min(c.W, X + c.R + 1);
        if (xh > x0 && xl < x0 + RAS_FSEG) {
            const float a = __int_as_float(en.x);
            for (int l = lane; l < P; l += 32) {
                const int x = xl + l;
                if (x < xh && x >= x0 && x < x0 + RAS_FSEG) buf[x - x0] = fmaf(a, A.cw[k * P + l], buf[x - x0]);
            }
        }
        __syncwarp();
    }
    const float4 p = b4[lane], q = b4[lane + 32];
    v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = p.w;
    v[4] = q.x; v[5] = q.y; v[6] = q.z; v[7] = q.w;
    __syncwarp();
}

template <bool VEC>
__global__ void __launch_bounds__(RAS_THREADS, 4)
raster_fast_kernel(const RasterConst c, const int64_t *__restrict__ off, const float4 *__restrict__ xyzi,
                   long long n_patterns, float *__restrict__ out, unsigned char *gscratch, size_t arena_bytes,
                   int32_t *status) {
    extern __shared__ __align__(16) unsigned char ras_smem[];
    unsigned char *base = gscratch ? gscratch + (size_t)blockIdx.x * arena_bytes : ras_smem;
    const int P = 2 * c.R + 1;
    const FastArena A = carve_fast(base, c.NS, c.T, c.H, P, c.one_pass ? fast_flag_bytes(c.H, c.W) : 0);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int H = c.H, W = c.W;
    const size_t img = (size_t)H * W;
    float *buf = A.rowbuf + warp * RAS_FSEG;

    for (long long p = blockIdx.x; p < n_patterns; p += gridDim.x) {
        const long long a0 = off[p];
        const long long n_ll = off[p + 1] - a0;
        if (n_ll > c.NS || n_ll < 0) {
            if (tid == 0) atomicOr(status, DS_ERR_CAPACITY);
            continue;
        }
        const int n = (int)n_ll;
        int Tp = 64;
        while (Tp < n + n / 2) Tp <<= 1;
        const int tbits = __ffs(Tp) - 1;
        for (int t = tid; t < Tp; t += RAS_THREADS) {
            A.hkey[t] = -1;
            A.hidx[t] = -1;
        }
        for (int y = tid; y <= H; y += RAS_THREADS) {
            A.rcnt[y] = 0;
            A.rfill[y] = 0;
        }
        if (tid == 0) A.misc[RAS_WARPS] = 0;
        __syncthreads();

        // ---- pixel coordinates, frame test, last write wins per pixel
        int my_in = 0;
        for (int i = tid; i < n; i += RAS_THREADS) {
            const float4 e = xyzi[a0 + i];
            int ix, iy;
            int key = -1, sl = -1;
            if (pixel_cell(c, e, ix, iy)) {
                ++my_in;
                key = iy * W + ix;
                // open addressing; Tp >= 1.5 n slots, so a free slot is always found
                unsigned h = ((unsigned)key * 2654435761u) >> (32 - tbits);
                for (int t = 0; t < Tp; ++t) {
                    const int prev = atomicCAS(&A.hkey[h], -1, key);
                    if (prev == -1 || prev == key) {
                        atomicMax(&A.hidx[h], i);
                        sl = (int)h;
                        break;
                    }
                    h = (h + 1) & (unsigned)(Tp - 1);
                }
                if (sl < 0) key = -1;
            }
            A.key[i] = key;
            A.slot[i] = sl;
        }
        my_in = __reduce_add_sync(FULL_MASK, my_in);
        if (lane == 0 && my_in) atomicAdd(&A.misc[RAS_WARPS], my_in);
        __syncthreads();
        const int n_in = A.misc[RAS_WARPS];

        // ---- ordered compaction, column weights, row counts
        int n_alive = 0;
        for (int c0 = 0; c0 < n; c0 += RAS_THREADS) {
            const int i = c0 + tid;
            bool alive = false;
            if (i < n && A.key[i] >= 0) alive = A.hidx[A.slot[i]] == i;
            const unsigned bal = __ballot_sync(FULL_MASK, alive);
            if (lane == 0) A.misc[warp] = __popc(bal);
            __syncthreads();
            int wbase = 0, tot = 0;
            for (int w = 0; w < RAS_WARPS; ++w) {
                const int v = A.misc[w];
                if (w < warp) wbase += v;
                tot += v;
            }
            if (alive) {
                const int k = n_alive + wbase + __popc(bal & ((1u << lane) - 1));
                const int key = A.key[i];
                const int X = key % W, Y = key / W;
                A.amp[k] = xyzi[a0 + i].w;
                A.sx[k] = X;
                A.sy[k] = Y;
                const int xlo = max(0, X - c.R), xhi = min(W, X + c.R + 1);
                for (int j = 0; j < xhi - xlo; ++j) A.cw[k * P + j] = reflect_weight(c, xlo + j, X, W);
                const int ylo = max(0, Y - c.R), yhi = min(H, Y + c.R + 1);
                for (int y = ylo; y < yhi; ++y) atomicAdd(&A.rcnt[y], 1);
            }
            n_alive += tot;
            __syncthreads();
        }

        // ---- row starts: exclusive scan of the counts over H + 1 entries
        {
            const int per = (H + 1 + RAS_THREADS - 1) / RAS_THREADS;
            const int y0 = tid * per, y1 = min(H + 1, y0 + per);
            int sum = 0;
            for (int y = y0; y < y1; ++y) sum += A.rcnt[y];
            const int inc = warp_inclusive_scan(sum, lane);
            if (lane == 31) A.misc[warp] = inc;
            __syncthreads();
            int run = inc - sum;
            for (int w = 0; w < warp; ++w) run += A.misc[w];
            for (int y = y0; y < y1; ++y) {
                A.rstart[y] = run;
                run += A.rcnt[y];
            }
            __syncthreads();
        }
        // ---- row entries (amp * row weight, X, spot), then each row's in spot order
        for (int k = tid; k < n_alive; k += RAS_THREADS) {
            const int X = A.sx[k], Y = A.sy[k];
            const float am = A.amp[k];
            const int ylo = max(0, Y - c.R), yhi = min(H, Y + c.R + 1);
            for (int y = ylo; y < yhi; ++y) {
                const int slot = A.rstart[y] + atomicAdd(&A.rfill[y], 1);
                if (DS_IN_BOUNDS(slot, (long long)c.NS * P, status))
                    A.ent[slot] = make_int2(__float_as_int(am * reflect_weight(c, y, Y, H)), (X << 16) | k);
            }
        }
        __syncthreads();
        for (int y = tid; y < H; y += RAS_THREADS) {
            const int e0 = A.rstart[y], e1 = A.rstart[y + 1];
            for (int e = e0 + 1; e < e1; ++e) {
                const int2 v = A.ent[e];
                const int kv = v.y & 0xffff;
                int f = e - 1;
                while (f >= e0 && (A.ent[f].y & 0xffff) > kv) {
                    A.ent[f + 1] = A.ent[f];
                    --f;
                }
                A.ent[f + 1] = v;
            }
        }
        __syncthreads();

        // ---- one pass (normalised, float4 rows): every covered row built once and
        // stored unscaled (the stores stay in L2), its non-zero float4 flagged;
        // then the maximum, and the flagged float4 rescaled in place (each lane
        // rereads only its own stores)
        if (VEC && c.one_pass && n_in > 0) {
            float *dst = out + (size_t)p * img;
            const int nseg = (W + RAS_FSEG - 1) / RAS_FSEG;
            float wm = -INFINITY;
            bool any_empty = false;
            for (int y = warp; y < H; y += RAS_WARPS) {
                float *row = dst + (size_t)y * W;
                if (A.rstart[y + 1] == A.rstart[y]) {
                    any_empty = true;
                    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
                    for (int x = lane * 4; x < W; x += 128) st_cs(reinterpret_cast<float4 *>(row + x), z);
                    continue;
                }
                for (int si = 0; si < nseg; ++si) {
                    const int x0 = si * RAS_FSEG;
                    float v[8];
                    fast_row_segment(c, A, P, y, x0, lane, buf, v);
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int xb = x0 + 128 * h + 4 * lane;
                        const bool in = xb < W;
                        const bool nz = in && (v[4 * h] != 0.f || v[4 * h + 1] != 0.f || v[4 * h + 2] != 0.f ||
                                               v[4 * h + 3] != 0.f);
                        if (in) {
                            st_wb(reinterpret_cast<float4 *>(row + xb),
                                  make_float4(v[4 * h], v[4 * h + 1], v[4 * h + 2], v[4 * h + 3]));
#pragma unroll
                            for (int e = 0; e < 4; ++e) wm = fmaxf(wm, v[4 * h + e]);
                        }
                        const unsigned bal = __ballot_sync(FULL_MASK, nz);
                        if (lane == 0) A.flags[((size_t)y * nseg + si) * 2 + h] = bal;
                    }
                }
            }
            if (any_empty) wm = fmaxf(wm, 0.f);
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) wm = fmaxf(wm, __shfl_xor_sync(FULL_MASK, wm, d));
            if (lane == 0) A.wmax[warp] = wm;
            __syncthreads();
            float mx = A.wmax[0];
            for (int w = 1; w < RAS_WARPS; ++w) mx = fmaxf(mx, A.wmax[w]);
            if (mx > 0.f && mx < INFINITY) {
                const float inv_mx = 1.f / mx;  // one reciprocal, then products (within 1 ulp of the quotients)
                for (int y = warp; y < H; y += RAS_WARPS) {
                    if (A.rstart[y + 1] == A.rstart[y]) continue;
                    float *row = dst + (size_t)y * W;
                    for (int si = 0; si < nseg; ++si) {
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const unsigned bal = A.flags[((size_t)y * nseg + si) * 2 + h];
                            if ((bal >> lane) & 1u) {
                                float4 *q = reinterpret_cast<float4 *>(row + si * RAS_FSEG + 128 * h + 4 * lane);
                                float4 t = *q;
                                t.x *= inv_mx; t.y *= inv_mx; t.z *= inv_mx; t.w *= inv_mx;
                                st_cs(q, t);
                            }
                        }
                    }
                }
            } else {
                // a maximum of zero, infinite or NaN: pattern / max everywhere, as numpy divides
                for (int y = warp; y < H; y += RAS_WARPS) {
                    float *row = dst + (size_t)y * W;
                    for (int x = lane * 4; x < W; x += 128) {
                        float4 *q = reinterpret_cast<float4 *>(row + x);
                        float4 t = *q;
                        t.x /= mx; t.y /= mx; t.z /= mx; t.w /= mx;
                        st_cs(q, t);
                    }
                }
            }
            __syncthreads();  // the arena is reused by the next pattern
            continue;
        }

        // ---- maximum over the image (normalise)
        float mx = 1.f;
        const bool norm = c.normalize && n_in > 0;
        if (norm) {
            float wm = -INFINITY;
            bool any_empty = false;
            for (int y = warp; y < H; y += RAS_WARPS) {
                if (A.rstart[y + 1] == A.rstart[y]) {
                    any_empty = true;
                    continue;
                }
                for (int x0 = 0; x0 < W; x0 += RAS_FSEG) {
                    float v[8];
                    fast_row_segment(c, A, P, y, x0, lane, buf, v);
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int x = x0 + (e < 4 ? 4 * lane + e : 128 + 4 * lane + e - 4);
                        if (x < W) wm = fmaxf(wm, v[e]);
                    }
                }
            }
            if (any_empty) wm = fmaxf(wm, 0.f);
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) wm = fmaxf(wm, __shfl_xor_sync(FULL_MASK, wm, d));
            if (lane == 0) A.wmax[warp] = wm;
            __syncthreads();
            mx = A.wmax[0];
            for (int w = 1; w < RAS_WARPS; ++w) mx = fmaxf(mx, A.wmax[w]);
        }

        // ---- the image
        float *dst = out + (size_t)p * img;
        const float zero_val = norm ? 0.f / mx : 0.f;
        // pattern / max: one reciprocal, then products (within 1 ulp of the quotients)
        const float inv_mx = norm ? 1.f / mx : 1.f;
        for (int y = warp; y < H; y += RAS_WARPS) {
            float *row = dst + (size_t)y * W;
            if (A.rstart[y + 1] == A.rstart[y]) {
                if (VEC) {
                    const float4 z = make_float4(zero_val, zero_val, zero_val, zero_val);
                    for (int x = lane * 4; x < W; x += 128) st_cs(reinterpret_cast<float4 *>(row + x), z);
                } else {
                    for (int x = lane; x < W; x += 32) st_cs1(row + x, zero_val);
                }
                continue;
            }
            for (int x0 = 0; x0 < W; x0 += RAS_FSEG) {
                float v[8];
                fast_row_segment(c, A, P, y, x0, lane, buf, v);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int xb = x0 + 128 * h + 4 * lane;
                    float s[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float u = v[4 * h + e];
                        s[e] = norm ? (u == 0.f ? zero_val : u * inv_mx) : u;
                    }
                    if (VEC) {
                        if (xb < W) st_cs(reinterpret_cast<float4 *>(row + xb), make_float4(s[0], s[1], s[2], s[3]));
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (xb + e < W) st_cs1(row + xb + e, s[e]);
                    }
                }
            }
        }
        __syncthreads();  // the arena is reused by the next pattern
    }
}

// ----------------------------------------------------------- slice mode ----
// Fast mode when the filter footprints and the per-pattern tables fit in
// shared memory (every detector up to a few thousand pixels wide).  The image
// is cut into slices of SH whole rows; warp w owns slices w, w + 8, ... and
// builds each one in a private shared-memory buffer, so no two warps ever
// touch the same pixel.  Each slice has the list of spots whose footprint
// reaches it, in ascending spot order; the warp takes the spots in that order
// and spreads a spot's footprint pixels (row, column pairs) over all 32 lanes,
// one fused multiply-add per pair.  A pair step never holds the same pixel
// twice, and the spots of one pixel are added in spot order: the image is
// deterministic, and equal across calls that split the patterns differently.
// Normalised images take two passes over the slices: the first finds the
// maximum (the running maximum of the updates when no amplitude is negative:
// the partial sums of non-negative terms never exceed their final value), the
// second rebuilds each slice and stores it scaled.  Global memory sees only the
// spot records and the image, written once.
#ifndef DS_RAS_SLICE_TARGET
#define DS_RAS_SLICE_TARGET (55 * 1024)  // shared bytes per CTA: four CTAs per SM
#endif
constexpr int RAS_SLICE_TARGET = DS_RAS_SLICE_TARGET;
static_assert(RAS_WARPS == 8, "slice ownership (s mod 8) assumes eight warps per CTA");

struct SliceGeom {
    int SH;      // rows per slice
    int Ws;      // buffer row stride in floats: >= W, a multiple of 4, = 4 ceil(P / 4) mod 32
    int nsl;     // slices per image
    int span;    // most slices one footprint reaches
    int P;       // footprint width 2R + 1
    unsigned mP; // ceil(2^32 / P): j / P = umulhi(j, mP) for j < P^2 (P odd, P^3 < 2^32)
    int wt2;     // the P x P product table is in shared memory (P <= 31)
    int loff;    // per-lane pair offsets in shared memory (wt2 and SH P <= 128)
};

struct SliceArena {
    float *buf;          // RAS_WARPS x SH x Ws
    int *key, *slot, *hkey, *hidx;
    int *sxy;            // X | Y << 15 | (footprint crosses an image edge) << 30
    float *amp;
    int *scnt, *sstart, *sfill;  // nsl + 1 each
    float *sU;                   // nsl + 1: a bound on every pixel of the slice (the maximum pass)
    int *sent;           // slice entries (spot indices), CSR by sstart
    float *wt, *wt2;     // 1-D weights w[|d|], d = 0..R; products w[|dy - R|] w[|dx - R|]
    int *loff;           // pair m -> (m / P) Ws + m % P, m < 128 (with g.loff)
    int *misc;
    float *wmax;
};

__host__ __device__ inline int slice_stride(int W, int P) {
    const int want = (4 * ((P + 3) / 4)) & 31;  // consecutive rows start 4 ceil(P / 4) banks apart
    return W + (((want - W) % 32) + 32) % 32;
}

__host__ __device__ inline size_t slice_arena_bytes(int NS, int T, int R, const SliceGeom &g) {
    size_t o = ras_align((size_t)RAS_WARPS * g.SH * g.Ws * 4);
    o += ras_align((size_t)NS * 4) * 2;              // key, slot
    o += ras_align((size_t)T * 4) * 2;               // hkey, hidx
    o += ras_align((size_t)NS * 4) * 2;              // sxy, amp
    o += ras_align((size_t)(g.nsl + 1) * 4) * 4;     // scnt, sstart, sfill, sU
    o += ras_align((size_t)NS * g.span * 4);         // sent
    o += ras_align((size_t)(R + 1) * 4);
    o += ras_align(g.wt2 ? (size_t)g.P * g.P * 4 : 0);
    o += ras_align(g.loff ? (size_t)128 * 4 : 0);
    o += ras_align(64 * 4) + ras_align(RAS_WARPS * 4);
    return o;
}

__device__ inline SliceArena carve_slice(unsigned char *base, int NS, int T, int R, const SliceGeom &g) {
    SliceArena A;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + o;
        o += ras_align(bytes);
        return p;
    };
    A.buf = (float *)take((size_t)RAS_WARPS * g.SH * g.Ws * 4);
    A.key = (int *)take((size_t)NS * 4);
    A.slot = (int *)take((size_t)NS * 4);
    A.hkey = (int *)take((size_t)T * 4);
    A.hidx = (int *)take((size_t)T * 4);
    A.sxy = (int *)take((size_t)NS * 4);
    A.amp = (float *)take((size_t)NS * 4);
    A.scnt = (int *)take((size_t)(g.nsl + 1) * 4);
    A.sstart = (int *)take((size_t)(g.nsl + 1) * 4);
    A.sfill = (int *)take((size_t)(g.nsl + 1) * 4);
    A.sU = (float *)take((size_t)(g.nsl + 1) * 4);
    A.sent = (int *)take((size_t)NS * g.span * 4);
    A.wt = (float *)take((size_t)(R + 1) * 4);
    A.wt2 = (float *)take(g.wt2 ? (size_t)g.P * g.P * 4 : 0);
    A.loff = (int *)take(g.loff ? (size_t)128 * 4 : 0);
    A.misc = (int *)take(64 * 4);
    A.wmax = (float *)take(RAS_WARPS * 4);
    return A;
}

// reflect_weight with the weights in shared memory
__device__ inline float reflect_weight_s(const float *wt, int R, int x, int P, int n) {
    float v = 0.f;
    if (R < n) {
        const int d = abs(x - P);
        if (d <= R) v += wt[d];
        const int m1 = x + P + 1;
        if (m1 <= R) v += wt[m1];
        const int m2 = 2 * n - 1 - P - x;
        if (m2 <= R) v += wt[m2];
        return v;
    }
    const int per = 2 * n;
    for (int fam = 0; fam < 2; ++fam) {
        const int base = fam == 0 ? P : -P - 1;
        const int k0 = (int)floor((double)(x - R - base) / per);
        for (int k = k0;; ++k) {
            const int q = base + k * per;
            if (q > x + R) break;
            if (q >= x - R) v += wt[abs(q - x)];
        }
    }
    return v;
}

// Adds the spots of slice rows [ys, ye) (entries e0..e1) into the warp's
// buffer; with TRACK, `run` takes the maximum of every updated value.
template <bool TRACK>
__device__ inline void slice_splat(const RasterConst &c, const SliceGeom &g, const SliceArena &A, int ys, int ye,
                                   int e0, int e1, float *buf, int lane, float &run, int32_t *status) {
    const int R = c.R, P = g.P, Ws = g.Ws;
    for (int e = e0; e < e1; ++e) {
        const int k = A.sent[e];
        const int v = A.sxy[k];
        const int X = v & 0x7fff, Y = (v >> 15) & 0x7fff;
        const float a = A.amp[k];
        const int y0 = max(Y - R, ys), y1 = min(Y + R + 1, ye);
        if (!(v >> 30) && g.loff) {
            // interior, pairs m of the footprint's rows y0..y1: weight
            // wt2[r0 P + m], buffer offset from the per-lane table
            const int jb = (y0 - (Y - R)) * P, np = (y1 - y0) * P;
            const int base = (y0 - ys) * Ws + (X - R);
            for (int m0 = 0; m0 < np; m0 += 32) {
                const int m = m0 + lane;
                if (m < np) {
                    const float w = A.wt2[jb + m];
                    const int o = base + A.loff[m];
                    if (!DS_IN_BOUNDS(o, (ye - ys) * Ws, status)) continue;
                    float *q = buf + o;
                    const float nv = fmaf(a, w, *q);
                    *q = nv;
                    if (TRACK) run = fmaxf(run, nv);
                }
            }
        } else if (!(v >> 30)) {
            // interior: pairs j = dy P + dx of the full footprint, rows y0..y1 only
            const int jb = (y0 - (Y - R)) * P, je = (y1 - (Y - R)) * P;
            const int corner = (Y - R - ys) * Ws + (X - R);  // footprint corner, relative to the slice (may be < 0)
            for (int j0 = jb; j0 < je; j0 += 32) {
                const int j = j0 + lane;
                if (j < je) {
                    const int dy = P == 1 ? j : (int)__umulhi((unsigned)j, g.mP);
                    const int dx = j - dy * P;
                    const float w = g.wt2 ? A.wt2[j] : A.wt[abs(dy - R)] * A.wt[abs(dx - R)];
                    if (!DS_IN_BOUNDS(corner + dy * Ws + dx, (ye - ys) * Ws, status)) continue;
                    float *q = buf + (corner + dy * Ws + dx);
                    const float nv = fmaf(a, w, *q);
                    *q = nv;
                    if (TRACK) run = fmaxf(run, nv);
                }
            }
        } else {
            // the footprint crosses an image edge: the clipped box, mirrored weights
            const int xl = max(0, X - R), xh = min(c.W, X + R + 1), nx = xh - xl;
            const int np = (y1 - y0) * nx;
            for (int j0 = 0; j0 < np; j0 += 32) {
                const int j = j0 + lane;
                if (j < np) {
                    const int dy = j / nx, dx = j - dy * nx;
                    const int y = y0 + dy, x = xl + dx;
                    const float w = reflect_weight_s(A.wt, R, y, Y, c.H) * reflect_weight_s(A.wt, R, x, X, c.W);
                    if (!DS_IN_BOUNDS((y - ys) * Ws + x, (ye - ys) * Ws, status)) continue;
                    float *q = buf + (y - ys) * Ws + x;
                    const float nv = fmaf(a, w, *q);
                    *q = nv;
                    if (TRACK) run = fmaxf(run, nv);
                }
            }
        }
        __syncwarp();
    }
}

__device__ inline void slice_zero(float *buf, int n_floats, int lane) {
    float4 *b4 = reinterpret_cast<float4 *>(buf);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = lane; i < n_floats / 4; i += 32) b4[i] = z;
    __syncwarp();
}

// pattern / max in float32: mode 0 multiplies by the reciprocal (max * (1 / max)
// == 1 exactly), mode 1 also returns 1 for the maximum itself, mode 2 divides
// (a maximum of zero, infinity or NaN, as numpy does)
template <int MODE>
__device__ __forceinline__ float slice_scale(float u, float mx, float inv) {
    if (MODE == 0) return u * inv;
    if (MODE == 1) return u == mx ? 1.f : u * inv;
    return u / mx;
}

constexpr int SLICE_FLAG_NEG = 1, SLICE_FLAG_NAN = 2;

template <bool VEC>
__global__ void __launch_bounds__(RAS_THREADS, 4)
raster_slice_kernel(const RasterConst c, const SliceGeom g, const int64_t *__restrict__ off,
                    const float4 *__restrict__ xyzi, long long n_patterns, float *__restrict__ out, int32_t *status) {
    extern __shared__ __align__(16) unsigned char ras_smem[];
    const int R = c.R, P = g.P, SH = g.SH, nsl = g.nsl;
    const SliceArena A = carve_slice(ras_smem, c.NS, c.T, R, g);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int H = c.H, W = c.W;
    const size_t img = (size_t)H * W;
    float *buf = A.buf + (size_t)warp * SH * g.Ws;
    const unsigned lt = (1u << lane) - 1u;

    for (int i = tid; i <= R; i += RAS_THREADS) A.wt[i] = c.wt[i];
    // a spot's largest pixel weight: w0^2 inside the image; at an edge each
    // axis adds at most three mirrored taps, or the whole filter (1) when
    // R >= the side
    const float w00 = c.wt[0] * c.wt[0];  // = the product table's centre entry
    const float wedge = (R < H && R < W) ? 9.f * w00 : 1.f;
    if (g.loff)
        for (int m = tid; m < 128; m += RAS_THREADS) A.loff[m] = (m / P) * g.Ws + m % P;
    // every slice build starts from a zero buffer: zeroed here once, then
    // cleaned by whoever used it (the read-back, or the maximum pass)
    slice_zero(buf, SH * g.Ws, lane);
    if (g.wt2)
        for (int j = tid; j < P * P; j += RAS_THREADS) {
            const int dy = j / P, dx = j - dy * P;
            A.wt2[j] = c.wt[abs(dy - R)] * c.wt[abs(dx - R)];
        }

    for (long long p = blockIdx.x; p < n_patterns; p += gridDim.x) {
        const long long a0 = off[p];
        const long long n_ll = off[p + 1] - a0;
        if (n_ll > c.NS || n_ll < 0) {
            if (tid == 0) atomicOr(status, DS_ERR_CAPACITY);
            continue;
        }
        const int n = (int)n_ll;
        int Tp = 64;
        while (Tp < n + n / 2) Tp <<= 1;
        const int tbits = __ffs(Tp) - 1;
        for (int t = tid; t < Tp; t += RAS_THREADS) {
            A.hkey[t] = -1;
            A.hidx[t] = -1;
        }
        for (int s = tid; s <= nsl; s += RAS_THREADS) {
            A.scnt[s] = 0;
            A.sfill[s] = 0;
            A.sU[s] = 0.f;
        }
        if (tid == 0) {
            A.misc[RAS_WARPS] = 0;      // in-frame spots
            A.misc[RAS_WARPS + 1] = 0;  // amplitude flags
            A.misc[RAS_WARPS + 2] = 0;  // largest non-negative amplitude (float bits)
        }
        __syncthreads();  // also orders the weight tables before their first use

        // ---- pixel coordinates, frame test, last write wins per pixel
        int my_in = 0;
        for (int i = tid; i < n; i += RAS_THREADS) {
            const float4 e = xyzi[a0 + i];
            int ix, iy;
            int key = -1, sl = -1;
            if (pixel_cell(c, e, ix, iy)) {
                ++my_in;
                key = iy * W + ix;
                unsigned h = ((unsigned)key * 2654435761u) >> (32 - tbits);
                for (int t = 0; t < Tp; ++t) {
                    const int prev = atomicCAS(&A.hkey[h], -1, key);
                    if (prev == -1 || prev == key) {
                        atomicMax(&A.hidx[h], i);
                        sl = (int)h;
                        break;
                    }
                    h = (h + 1) & (unsigned)(Tp - 1);
                }
                if (sl < 0) key = -1;
            }
            A.key[i] = key;
            A.slot[i] = sl;
        }
        my_in = __reduce_add_sync(FULL_MASK, my_in);
        if (lane == 0 && my_in) atomicAdd(&A.misc[RAS_WARPS], my_in);
        __syncthreads();
        const int n_in = A.misc[RAS_WARPS];

        // ---- ordered compaction, slice counts, amplitude flags
        int n_alive = 0;
        for (int c0 = 0; c0 < n; c0 += RAS_THREADS) {
            const int i = c0 + tid;
            bool alive = false;
            if (i < n && A.key[i] >= 0) alive = A.hidx[A.slot[i]] == i;
            const unsigned bal = __ballot_sync(FULL_MASK, alive);
            if (lane == 0) A.misc[warp] = __popc(bal);
            __syncthreads();
            int wbase = 0, tot = 0;
            for (int w = 0; w < RAS_WARPS; ++w) {
                const int v = A.misc[w];
                if (w < warp) wbase += v;
                tot += v;
            }
            if (alive) {
                const int k = n_alive + wbase + __popc(bal & lt);
                const int key = A.key[i];
                const int X = key % W, Y = key / W;
                const float am = xyzi[a0 + i].w;
                const bool edge = X - R < 0 || X + R >= W || Y - R < 0 || Y + R >= H;
                A.sxy[k] = X | (Y << 15) | ((int)edge << 30);
                A.amp[k] = am;
                if (!(am >= 0.f)) atomicOr(&A.misc[RAS_WARPS + 1], am != am ? SLICE_FLAG_NAN : SLICE_FLAG_NEG);
                else atomicMax(&A.misc[RAS_WARPS + 2], __float_as_int(am));  // non-negative floats order as ints
                const int s0 = max(0, Y - R) / SH, s1 = min(H - 1, Y + R) / SH;
                // the slices' pixel bounds (in any order: a bound, widened below)
                const float ub = am * (edge ? wedge : w00);
                for (int s = s0; s <= s1; ++s) {
                    atomicAdd(&A.scnt[s], 1);
                    atomicAdd(&A.sU[s], ub);
                }
            }
            n_alive += tot;
            __syncthreads();
        }
        const int aflags = A.misc[RAS_WARPS + 1];

        // ---- slice starts: exclusive scan of the counts over nsl + 1 entries
        {
            const int per = (nsl + 1 + RAS_THREADS - 1) / RAS_THREADS;
            const int s0 = tid * per, s1 = min(nsl + 1, s0 + per);
            int sum = 0;
            for (int s = s0; s < s1; ++s) sum += A.scnt[s];
            const int inc = warp_inclusive_scan(sum, lane);
            if (lane == 31) A.misc[warp] = inc;
            __syncthreads();
            int run = inc - sum;
            for (int w = 0; w < warp; ++w) run += A.misc[w];
            for (int s = s0; s < s1; ++s) {
                A.sstart[s] = run;
                run += A.scnt[s];
            }
            __syncthreads();
        }

        // ---- slice entries in spot order: warp w fills its own slices, 32 spots
        // at a time; within a slice the lanes take consecutive places by lane.
        // When a footprint spans at most 8 slices a spot has at most one slice
        // of each warp: one match over the lanes' slices places them all.
        for (int k0 = 0; g.span <= 8 && k0 < n_alive; k0 += 32) {
            const int k = k0 + lane;
            int s = -1;
            if (k < n_alive) {
                const int Y = (A.sxy[k] >> 15) & 0x7fff;
                const int s0 = max(0, Y - R) / SH, s1 = min(H - 1, Y + R) / SH;
                const int f = s0 + ((warp - s0) & 7);  // the warp's slice in [s0, s1], if any
                if (f <= s1) s = f;
            }
            const unsigned grp = __match_any_sync(FULL_MASK, s);
            if (s >= 0) {
                const int place = A.sstart[s] + A.sfill[s] + __popc(grp & lt);
                if (DS_IN_BOUNDS(place, (long long)c.NS * g.span, status)) A.sent[place] = k;
            }
            __syncwarp();
            if (s >= 0 && (grp >> lane) == 1u) A.sfill[s] += __popc(grp);  // the group's last lane
            __syncwarp();
        }
        for (int k0 = 0; g.span > 8 && k0 < n_alive; k0 += 32) {
            const int k = k0 + lane;
            int t0 = 1 << 30, t1 = -(1 << 30);
            if (k < n_alive) {
                const int Y = (A.sxy[k] >> 15) & 0x7fff;
                const int s0 = max(0, Y - R) / SH, s1 = min(H - 1, Y + R) / SH;
                const int f = s0 + ((warp - s0) & 7), l = s1 - ((s1 - warp) & 7);  // owned slices in [s0, s1]
                t0 = (f - warp) >> 3;
                t1 = (l - warp) >> 3;
            }
            const int tmin = __reduce_min_sync(FULL_MASK, t0), tmax = __reduce_max_sync(FULL_MASK, t1);
            for (int t = tmin; t <= tmax; ++t) {
                const bool act = t0 <= t && t <= t1;
                const unsigned bal = __ballot_sync(FULL_MASK, act);
                if (!bal) continue;
                const int s = warp + 8 * t;
                const int base = A.sstart[s] + A.sfill[s];
                if (act && DS_IN_BOUNDS(base + __popc(bal & lt), (long long)c.NS * g.span, status))
                    A.sent[base + __popc(bal & lt)] = k;
                __syncwarp();
                if (lane == 0) A.sfill[s] += __popc(bal);
                __syncwarp();
            }
        }
        __syncthreads();

        // ---- the maximum (normalise).  Without negative amplitudes only the
        // slices that can hold it are built: the centre pixel of the strongest
        // spot is at least lower = a_max w0^2 (its other terms are >= 0, and a
        // rounded non-negative sum never falls below a term), and no pixel of
        // a slice exceeds its bound U = sum of a_k times the spot's largest
        // weight (w0^2 inside the image; at an edge each axis adds at most
        // three mirrored taps, or the whole filter, 1, when R >= the side),
        // widened by 0.1 % for rounding.  A slice with U < lower is skipped.
        const bool norm = c.normalize && n_in > 0;
        float mx = 1.f;
        if (norm) {
            const bool readback = (aflags & SLICE_FLAG_NEG) != 0;
            const float lower = __int_as_float(A.misc[RAS_WARPS + 2]) * w00;
            float run = -INFINITY;
            bool any_empty = false;
            for (int s = warp; s < nsl; s += RAS_WARPS) {
                const int e0 = A.sstart[s], e1 = A.sstart[s + 1];
                if (e0 == e1) {
                    any_empty = true;
                    continue;
                }
                // the bound summed in compaction (atomics: any order; the 0.1 %
                // covers its rounding up to ~1.6e4 spots per slice)
                if (!readback && A.sU[s] * 1.001f < lower) continue;
                const int ys = s * SH, ye = min(H, ys + SH);
                if (readback) {
                    slice_splat<false>(c, g, A, ys, ye, e0, e1, buf, lane, run, status);
                    for (int r = 0; r < ye - ys; ++r)
                        for (int x = lane; x < W; x += 32) run = fmaxf(run, buf[r * g.Ws + x]);
                    __syncwarp();
                } else {
                    slice_splat<true>(c, g, A, ys, ye, e0, e1, buf, lane, run, status);
                }
                slice_zero(buf, (ye - ys) * g.Ws, lane);  // clean for the next build
            }
            // without negative amplitudes every pixel is >= 0, uncovered ones 0
            if (any_empty || !readback) run = fmaxf(run, 0.f);
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) run = fmaxf(run, __shfl_xor_sync(FULL_MASK, run, d));
            if (lane == 0) A.wmax[warp] = run;
            __syncthreads();
            mx = A.wmax[0];
            for (int w = 1; w < RAS_WARPS; ++w) mx = fmaxf(mx, A.wmax[w]);
            if (aflags & SLICE_FLAG_NAN) mx = NAN;  // numpy's max propagates NaN
        }
        const float inv = 1.f / mx;
        const int mode = !norm ? 0 : !(mx > 0.f && mx < INFINITY) ? 2 : mx * inv == 1.f ? 0 : 1;
        const float sc_inv = norm ? inv : 1.f;
        const float zero_val = norm ? 0.f / mx : 0.f;

        // ---- the image, slice by slice
        float *dst0 = out + (size_t)p * img;
        for (int s = warp; s < nsl; s += RAS_WARPS) {
            const int ys = s * SH, ye = min(H, ys + SH);
            float *dst = dst0 + (size_t)ys * W;
            const int e0 = A.sstart[s], e1 = A.sstart[s + 1];
            if (e0 == e1) {
                const int nf = (ye - ys) * W;
                if (VEC) {
                    const float4 z = make_float4(zero_val, zero_val, zero_val, zero_val);
                    for (int i = lane; i < nf / 4; i += 32) st_cs(reinterpret_cast<float4 *>(dst) + i, z);
                } else {
                    for (int i = lane; i < nf; i += 32) st_cs1(dst + i, zero_val);
                }
                continue;
            }
            float unused = 0.f;
            slice_splat<false>(c, g, A, ys, ye, e0, e1, buf, lane, unused, status);
            // read back, scale, store; zeros written back leave the buffer clean
            auto store_rows = [&](auto md) {
                constexpr int MODE = decltype(md)::value;
                for (int r = 0; r < ye - ys; ++r) {
                    float *src = buf + r * g.Ws;
                    float *row = dst + (size_t)r * W;
                    if (VEC) {
                        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
                        for (int x = 4 * lane; x < W; x += 128) {
                            float4 *q = reinterpret_cast<float4 *>(src + x);
                            const float4 u = *q;
                            *q = z4;
                            st_cs(reinterpret_cast<float4 *>(row + x),
                                  make_float4(slice_scale<MODE>(u.x, mx, sc_inv), slice_scale<MODE>(u.y, mx, sc_inv),
                                              slice_scale<MODE>(u.z, mx, sc_inv), slice_scale<MODE>(u.w, mx, sc_inv)));
                        }
                    } else {
                        for (int x = lane; x < W; x += 32) {
                            const float u = src[x];
                            src[x] = 0.f;
                            st_cs1(row + x, slice_scale<MODE>(u, mx, sc_inv));
                        }
                    }
                }
            };
            if (mode == 0) store_rows(std::integral_constant<int, 0>{});
            else if (mode == 1) store_rows(std::integral_constant<int, 1>{});
            else store_rows(std::integral_constant<int, 2>{});
            __syncwarp();
        }
        __syncthreads();  // the arena is reused by the next pattern
    }
}

static bool slice_geometry(const ds_raster_params *p, int NS, int T, int R, SliceGeom &g, size_t &bytes) {
    const int H = p->height, W = p->width, P = 2 * R + 1;
    if (!p->fast || W >= (1 << 15) || H >= (1 << 15)) return false;
    for (int SH : {8, 4, 2, 1}) {
        g.SH = SH;
        g.P = P;
        g.Ws = slice_stride(W, P);
        g.nsl = (H + SH - 1) / SH;
        g.span = std::min(g.nsl, (P - 1 + SH - 1) / SH + 1);
        g.mP = P > 1 ? (unsigned)((0x100000000ull + P - 1) / P) : 0u;
        g.wt2 = P <= 31 ? 1 : 0;
        g.loff = (g.wt2 && SH * P <= 128) ? 1 : 0;
        bytes = slice_arena_bytes(NS, T, R, g);
        if (bytes <= (size_t)RAS_SLICE_TARGET || (SH == 1 && bytes <= RAS_SMEM_LIMIT)) return true;
    }
    return false;
}

struct RasterPlan {
    int NS, T, grid;
    bool one_pass, slice;
    SliceGeom g;
    size_t arena, smem, scratch;
};

static int filter_radius(const ds_raster_params *p) {
    return (p->fast && p->sigma > 1e-15) ? (int)(p->truncate * p->sigma + 0.5) : 0;
}

template <bool VEC>
static const void *raster_kernel_ptr(bool fast) {
    return fast ? (const void *)raster_fast_kernel<VEC> : (const void *)raster_kernel<VEC>;
}

static ds_status raster_plan(const ds_raster_params *p, int64_t max_spots, RasterPlan &P) {
    DS_REQUIRE(max_spots >= 0 && max_spots < (1ll << 28), "ds_rasterize: max_spots out of range");
    DS_REQUIRE(!p->fast || max_spots <= 65504, "ds_rasterize: at most 65504 spots per pattern in fast mode");
    int NS = (int)std::max<int64_t>(32, (max_spots + 31) / 32 * 32);
    const bool fast = p->fast != 0;
    int T = 64;
    while (fast ? T < NS + NS / 2 : T < 2 * NS) T <<= 1;  // the kernels' per-pattern hash sizes
    P.NS = NS;
    P.T = T;
    int dev = 0, n_sm = 0;
    DS_CUDA_TRY(cudaGetDevice(&dev));
    DS_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    size_t slice_bytes = 0;
    P.slice = slice_geometry(p, NS, T, filter_radius(p), P.g, slice_bytes);
    if (P.slice) {
        P.one_pass = false;
        P.arena = P.smem = slice_bytes;
        P.scratch = 0;
        int per_sm = 0;
        for (const void *k : {(const void *)raster_slice_kernel<true>, (const void *)raster_slice_kernel<false>})
            DS_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem));
        DS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, raster_slice_kernel<true>, RAS_THREADS,
                                                                  P.smem));
        P.grid = n_sm * std::max(1, per_sm);
        return DS_OK;
    }
    P.one_pass = fast && p->normalize && (p->width % 4) == 0 && fast_flag_bytes(p->height, p->width) <= RAS_FLAGS_MAX;
    P.arena = fast ? fast_arena_bytes(NS, T, p->height, 2 * filter_radius(p) + 1,
                                      P.one_pass ? fast_flag_bytes(p->height, p->width) : 0)
                   : raster_arena_bytes(NS, T, p->height);
    if (P.arena <= RAS_SMEM_LIMIT) {
        P.smem = P.arena;
        P.scratch = 0;
        int per_sm = 0;
        for (const void *k : {raster_kernel_ptr<true>(fast), raster_kernel_ptr<false>(fast)})
            DS_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem));
        DS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, raster_kernel_ptr<true>(fast), RAS_THREADS,
                                                                  P.smem));
        P.grid = n_sm * std::max(1, per_sm);
    } else {
        P.smem = 0;
        P.grid = 2 * n_sm;
        P.scratch = (size_t)P.grid * P.arena;
    }
    return DS_OK;
}

static ds_status raster_validate(const ds_raster_params *p) {
    DS_REQUIRE(p, "ds_rasterize: null params");
    DS_REQUIRE(p->height > 0 && p->width > 0 && p->height <= 32768 && p->width <= 32768,
               "ds_rasterize: shape must be 1..32768 pixels per side");
    DS_REQUIRE((long long)p->height * p->width < (1ll << 31), "ds_rasterize: image too large");
    DS_REQUIRE(std::isfinite(p->calibration) && p->calibration != 0.0, "ds_rasterize: calibration must be finite, non-zero");
    DS_REQUIRE(std::isfinite(p->center_x) && std::isfinite(p->center_y) && std::isfinite(p->in_plane_angle),
               "ds_rasterize: centre and angle must be finite");
    DS_REQUIRE(std::isfinite(p->sigma), "ds_rasterize: sigma must be finite");
    DS_REQUIRE(p->pixel_snap >= 0.0 && p->pixel_snap < 0.5, "ds_rasterize: pixel_snap must be in [0, 0.5)");
    if (p->fast) {
        DS_REQUIRE(std::isfinite(p->truncate) && p->truncate >= 0.0, "ds_rasterize: truncate must be >= 0");
        if (p->sigma > 1e-15) {
            const double r = p->truncate * p->sigma + 0.5;
            DS_REQUIRE(r < RAS_MAX_R + 1, "ds_rasterize: filter radius int(truncate * sigma + 0.5) must be <= 511");
        }
    } else {
        DS_REQUIRE(p->sigma != 0.0, "ds_rasterize: sigma must be non-zero in sub-pixel mode");
        DS_REQUIRE(!std::isnan(p->clip_threshold), "ds_rasterize: clip_threshold is NaN");
    }
    return DS_OK;
}

}  // namespace ds

using namespace ds;

extern "C" size_t ds_rasterize_scratch_bytes(const ds_raster_params *p, int64_t max_spots) {
    clear_error();
    if (raster_validate(p) != DS_OK) return 0;
    RasterPlan P;
    if (raster_plan(p, max_spots, P) != DS_OK) return 0;
    return P.scratch;
}

extern "C" ds_status ds_rasterize(const ds_raster_params *p, const int64_t *offsets, const float *xyzi,
                                  int64_t n_patterns, int64_t max_spots, float *out, void *scratch,
                                  size_t scratch_bytes, int32_t *status, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_rasterize");
    ds_status st = raster_validate(p);
    if (st) return st;
    DS_REQUIRE(status, "ds_rasterize: null status");
    DS_REQUIRE(n_patterns >= 0, "ds_rasterize: n_patterns < 0");
    if (n_patterns == 0) return DS_OK;
    DS_REQUIRE(offsets && out, "ds_rasterize: null offsets / out");
    DS_REQUIRE(xyzi || max_spots == 0, "ds_rasterize: null xyzi");
    DS_REQUIRE(((uintptr_t)xyzi & 15) == 0, "ds_rasterize: xyzi must be 16-byte aligned");
    const bool vec = (p->width % 4) == 0 && ((uintptr_t)out & 15) == 0;
    RasterPlan P;
    st = raster_plan(p, max_spots, P);
    if (st) return st;
    DS_REQUIRE(P.scratch == 0 || (scratch && scratch_bytes >= P.scratch), "ds_rasterize: scratch too small");

    RasterConst c;
    c.H = p->height;
    c.W = p->width;
    c.fast = p->fast ? 1 : 0;
    c.normalize = p->normalize ? 1 : 0;
    c.NS = P.NS;
    c.T = P.T;
    c.one_pass = P.one_pass && vec ? 1 : 0;
    c.cal = p->calibration;
    c.cx = p->center_x;
    c.cy = p->center_y;
    const double PI = 3.14159265358979323846;
    const double th = p->in_plane_angle * (PI / 180.0);  // numpy.deg2rad
    c.ca = cos(th);
    c.sa = sin(th);
    c.mf = p->mirrored ? -1.0 : 1.0;
    c.snap = p->pixel_snap;
    c.icf = (float)(1.0 / c.cal);
    c.caf = (float)c.ca;
    c.saf = (float)c.sa;
    c.mff = (float)c.mf;
    c.cxf = (float)c.cx;
    c.cyf = (float)c.cy;
    c.snapf = (float)c.snap;
    c.clip = p->clip_threshold;
    c.pref = 1.0 / (2.0 * PI * p->sigma * p->sigma);
    c.exp_pref = -1.0 / (2.0 * p->sigma * p->sigma);
    for (int i = 0; i <= RAS_MAX_R; ++i) c.wt[i] = 0.f;
    c.R = 0;
    if (c.fast) {
        if (p->sigma > 1e-15) {
            // scipy.ndimage._gaussian_kernel1d: exp(-0.5 / sigma^2 x^2), normalised
            const int R = (int)(p->truncate * p->sigma + 0.5);
            const double s2 = p->sigma * p->sigma;
            double phi[RAS_MAX_R + 1], sum = 0.0;
            for (int x = 0; x <= R; ++x) phi[x] = exp(-0.5 / s2 * (double)x * (double)x);
            for (int x = -R; x <= R; ++x) sum += phi[x < 0 ? -x : x];
            for (int x = 0; x <= R; ++x) c.wt[x] = (float)(phi[x] / sum);
            c.R = R;
        } else {
            c.wt[0] = 1.f;  // the filter is skipped for sigma <= 1e-15
        }
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int grid = (int)std::min<long long>(P.grid, n_patterns);
    unsigned char *g = P.scratch ? reinterpret_cast<unsigned char *>(scratch) : nullptr;
    const float4 *x4 = reinterpret_cast<const float4 *>(xyzi);
    size_t arena = P.arena;
    long long np = n_patterns;
    if (P.slice) {
        SliceGeom geo = P.g;
        void *sargs[] = {&c, &geo, const_cast<int64_t **>(&offsets), const_cast<float4 **>(&x4), &np, &out, &status};
        const void *kern = vec ? (const void *)raster_slice_kernel<true> : (const void *)raster_slice_kernel<false>;
        DS_CUDA_TRY(cudaLaunchKernel(kern, dim3(grid), dim3(RAS_THREADS), sargs, P.smem, s));
        return check_launch("raster_slice_kernel");
    }
    void *args[] = {&c, const_cast<int64_t **>(&offsets), const_cast<float4 **>(&x4), &np, &out, &g, &arena, &status};
    const void *kern = vec ? raster_kernel_ptr<true>(c.fast != 0) : raster_kernel_ptr<false>(c.fast != 0);
    DS_CUDA_TRY(cudaLaunchKernel(kern, dim3(grid), dim3(RAS_THREADS), args, P.smem, s));
    return check_launch(c.fast ? "raster_fast_kernel" : "raster_kernel");
}
