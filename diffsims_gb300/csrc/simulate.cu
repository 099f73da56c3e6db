// A4-A7 host side: launch plan, scratch layout and the ds_simulate entry
// point of the orientation kernel (device code in simulate_kernel.cuh).
#include <algorithm>

#include "simulate_kernel.cuh"

namespace ds {

// ------------------------------------------------------------------ prep ----
// Per row: (h, k, l, -z_mid) and z_half of the z-interval that holds every
// selected (orientation, row) pair, plus |g|^2 as a float pair.
// |s| < e  <=>  z_a < z < z_b with z_a = (g^2 + e^2 - 2 e k0) / (2 (k0 - e)),
// z_b = (g^2 + e^2 + 2 e k0) / (2 (k0 + e))  (s is decreasing in z).
// For precession e is widened by a bound on how far the precessing sphere
// strays from the static one at this |g|:
//   k0 (1 - cos phi) + Pt (2 |g| + Pt) / (2 sqrt(k0^2 - (|g| + Pt)^2)).
__global__ void sim_prep_kernel(SimConst c, const int32_t *__restrict__ hkl, const double *__restrict__ g2,
                                const float *__restrict__ F2, float4 *__restrict__ scr, float *__restrict__ zh,
                                float4 *__restrict__ aux) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= c.n_hkl) return;
    double gsq = g2[j];
    double e = c.eps;
    if (c.prec != DS_PRECESSION_NONE) {
        double g = sqrt(gsq);
        double a = c.k0 * c.k0 - (g + c.Pt) * (g + c.Pt);
        double wide = a > 0 ? c.k0 * (1.0 - cos(c.phi)) + c.Pt * (2.0 * g + c.Pt) / (2.0 * sqrt(a)) : 1e30;
        e = c.eps + wide * 1.0001 + 1e-7;
    }
    double za = (gsq + e * e - 2.0 * e * c.k0) / (2.0 * (c.k0 - e));
    double zb = (gsq + e * e + 2.0 * e * c.k0) / (2.0 * (c.k0 + e));
    double zmid = 0.5 * (za + zb), zhalf = 0.5 * (zb - za);
    const float4 row = make_float4((float)hkl[3 * j], (float)hkl[3 * j + 1], (float)hkl[3 * j + 2], (float)(-zmid));
    scr[j] = row;
    zh[j] = (float)zhalf + c.guard;
    float hi, lo;
    split_double(gsq, hi, lo);
    aux[2 * j] = row;
    aux[2 * j + 1] = make_float4(hi, lo, F2 ? F2[j] : 0.f, 0.f);
}

__global__ void __launch_bounds__(LN_THREADS)
lines_kernel(SimConst c, const int32_t *__restrict__ hkl, LineP *__restrict__ lines, int *__restrict__ meta,
             LookbackScratch lb, long long n_tiles, int32_t *status) {
    // meta[0] = number of lines, meta[1] = first trailing 000 row
    __shared__ long long s_tile, s_prefix;
    __shared__ int s_warp[LN_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = (long long)atomicAdd(lb.ticket, 1ull);
    __syncthreads();
    const long long tile = s_tile;
    const long long base = tile * LN_TILE + (long long)tid * LN_ITEMS;
    bool start[LN_ITEMS];
    int cnt = 0;
#pragma unroll
    for (int it = 0; it < LN_ITEMS; ++it) {
        const long long j = base + it;
        start[it] = false;
        if (j < c.n_hkl) {
            if (row_is_zero(hkl, j)) {
                atomicMin(&meta[1], (int)j);
            } else {
                // a line is a run of equal (h, k) with consecutive l; the (0, 0) run
                // is split at the missing 000 row
                start[it] = j == 0 || hkl[3 * j - 3] != hkl[3 * j] || hkl[3 * j - 2] != hkl[3 * j + 1] ||
                            hkl[3 * j - 1] != hkl[3 * j + 2] + 1;
            }
        }
        cnt += start[it] ? 1 : 0;
    }
    const int incl = warp_inclusive_scan(cnt, lane);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int v = lane < LN_THREADS / 32 ? s_warp[lane] : 0;
        const int w = warp_inclusive_scan(v, lane);
        if (lane < LN_THREADS / 32) s_warp[lane] = w - v;
        if (lane == LN_THREADS / 32 - 1) {
            const long long prefix = lookback_exclusive(lb, tile, (long long)w, status);
            s_prefix = prefix;
            if (prefix >= 0 && tile == n_tiles - 1) meta[0] = (int)(prefix + w);
        }
    }
    __syncthreads();
    if (s_prefix < 0) return;
    long long pos = s_prefix + s_warp[warp] + (incl - cnt);
#pragma unroll
    for (int it = 0; it < LN_ITEMS; ++it) {
        if (!start[it]) continue;
        const long long j = base + it;
        const int h = hkl[3 * j], k = hkl[3 * j + 1];
        long long e = j + 1;
        while (e < c.n_hkl && hkl[3 * e] == h && hkl[3 * e + 1] == k && hkl[3 * e + 2] == hkl[3 * e - 1] - 1 &&
               !row_is_zero(hkl, e))
            ++e;
        // P, Q in FP64 from the reciprocal basis (rows a*, b*, c*)
        double v[3];
        for (int t = 0; t < 3; ++t) v[t] = (double)h * c.recip[t] + (double)k * c.recip[3 + t];
        const double P = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        const double Q = v[0] * c.recip[6] + v[1] * c.recip[7] + v[2] * c.recip[8];
        LineP L;
        L.h = (float)h;
        L.k = (float)k;
        L.pa = (float)(c.alpha0 - (double)c.guard + c.alpha1 * P);
        L.qa = (float)(2.0 * c.alpha1 * Q);
        L.pb = (float)(c.beta0 + (double)c.guard + c.beta1 * P);
        L.qb = (float)(2.0 * c.beta1 * Q);
        L.row0 = (int)j;
        L.n = (int)(e - j);
        L.l_top = hkl[3 * j + 2];
        L.kc = fabsf(L.pa) + fabsf(L.pb);
        L.kq = fabsf(L.qa) + fabsf(L.qb);
        L.lmax = (float)max(abs(L.l_top), abs(L.l_top - L.n + 1));
        lines[pos] = L;
        ++pos;
    }
}

static inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// ---------------------------------------------------------------- bricks ----
// Rows per block (atomic counts).
__global__ void brick_count_kernel(BrickGeom G, const int32_t *__restrict__ hkl, long long n, int32_t *cnt) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    atomicAdd(&cnt[brick_block(G, hkl[3 * j], hkl[3 * j + 1], hkl[3 * j + 2])], 1);
}

// One block: each block of rows becomes ceil(count / 32) bricks of 32 slots;
// first[blk] = its first brick (exclusive scan), bblk[brick] = its block,
// meta[0] = number of bricks.
constexpr int BRICK_SCAN_THREADS = 1024;
__global__ void __launch_bounds__(BRICK_SCAN_THREADS)
brick_scan_kernel(int nblk, const int32_t *__restrict__ cnt, int32_t *first, int32_t *bblk, int32_t *meta) {
    __shared__ int s_part[BRICK_SCAN_THREADS / 32];
    __shared__ int s_carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_carry = 0;
    __syncthreads();
    for (int i0 = 0; i0 < nblk; i0 += BRICK_SCAN_THREADS) {
        const int i = i0 + tid;
        const int v = i < nblk ? (cnt[i] + 31) / 32 : 0;
        const int iv = warp_inclusive_scan(v, lane);
        if (lane == 31) s_part[warp] = iv;
        __syncthreads();
        if (warp == 0) {
            const int a = s_part[lane];
            s_part[lane] = warp_inclusive_scan(a, lane) - a;
        }
        __syncthreads();
        const int f = s_carry + s_part[warp] + iv - v;
        if (i < nblk) {
            first[i] = f;
            for (int k = 0; k < v; ++k) bblk[f + k] = i;
        }
        __syncthreads();
        if (tid == BRICK_SCAN_THREADS - 1) s_carry = f + v;
        __syncthreads();
    }
    if (tid == 0) meta[0] = s_carry;
}

// Rows into the slots of their block's bricks, with copies of their screen
// data (the order inside a block is immaterial: the screen sets bits at the
// rows' table positions).
__global__ void brick_fill_kernel(BrickGeom G, const int32_t *__restrict__ hkl, long long n,
                                  const int32_t *__restrict__ first, int32_t *fill, const float4 *__restrict__ scr,
                                  const float *__restrict__ zh, int32_t *bperm, float4 *bscr, float *bzh) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int blk = brick_block(G, hkl[3 * j], hkl[3 * j + 1], hkl[3 * j + 2]);
    const long long slot = 32ll * first[blk] + atomicAdd(&fill[blk], 1);
    bperm[slot] = (int32_t)j;
    bscr[slot] = scr[j];
    bzh[slot] = zh[j];
}

// One warp per brick: the empty slots filled (row -1, z_half -1: never
// passes), the band [lo, hi] of the rows' z-intervals (the prep's FP32
// values, as the row test uses them) and the block centre.
__global__ void brick_bounds_kernel(BrickGeom G, const int32_t *__restrict__ bblk, const int32_t *__restrict__ first,
                                    const int32_t *__restrict__ cnt, const int32_t *__restrict__ meta, int32_t *bperm,
                                    float4 *bscr, float *bzh, float4 *brec, float *bhalf) {
    const int lane = threadIdx.x & 31;
    const long long b = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= meta[0]) return;
    const int blk = bblk[b];
    const int in_brick = min(32, cnt[blk] - 32 * (int)(b - first[blk]));
    const long long slot = 32 * b + lane;
    float lo = INFINITY, hi = -INFINITY;
    if (lane < in_brick) {
        const float zm = -bscr[slot].w, w = bzh[slot];
        lo = zm - w;
        hi = zm + w;
    } else {
        bperm[slot] = -1;
        bscr[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
        bzh[slot] = -1.f;
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(FULL_MASK, lo, d));
        hi = fmaxf(hi, __shfl_xor_sync(FULL_MASK, hi, d));
    }
    if (lane == 0) {
        const int bz = blk % G.nbz, by = (blk / G.nbz) % G.nby, bx = blk / (G.nbz * G.nby);
        const float hc = (float)(bx * G.bh - G.hmax[0]) + 0.5f * (float)(G.bh - 1);
        const float kc = (float)(by * G.bk - G.hmax[1]) + 0.5f * (float)(G.bk - 1);
        const float lc = (float)(bz * G.bl - G.hmax[2]) + 0.5f * (float)(G.bl - 1);
        brec[b] = make_float4(hc, kc, lc, -0.5f * (lo + hi));
        bhalf[b] = 0.5f * (hi - lo) + G.rho_margin;
    }
}

BrickGeom brick_geometry(const double recip[9], const int32_t hmax[3], int O, double reach) {
    // cost per row and tile ~ (C0 + O C1 pass) / P for bricks of P rows, the
    // pass rate ~ the share of a ball of radius R within rho + reach of a
    // plane through its centre: 1.5 (rho + reach) / R
    double len[3], R = 0.0;
    for (int i = 0; i < 3; ++i) {
        len[i] = sqrt(recip[3 * i] * recip[3 * i] + recip[3 * i + 1] * recip[3 * i + 1] +
                      recip[3 * i + 2] * recip[3 * i + 2]);
        R = fmax(R, len[i] * (double)(hmax[i] > 0 ? hmax[i] : 1));
    }
    const double C0 = 12.0, C1 = 11.0;
    BrickGeom G{};
    double best = 1e300, best_rho = 0.0;
    for (int bh = 1; bh <= 8; ++bh)
        for (int bk = 1; bk <= 8; ++bk)
            for (int bl = 1; bl <= 8; ++bl) {
                const int P = bh * bk * bl;
                if (P > 32) continue;
                double rho = 0.0;  // the largest corner of the block, |B*^T (d_h, d_k, d_l)|
                for (int sh = -1; sh <= 1; sh += 2)
                    for (int sk = -1; sk <= 1; sk += 2)
                        for (int sl = -1; sl <= 1; sl += 2) {
                            const double d[3] = {0.5 * sh * (bh - 1), 0.5 * sk * (bk - 1), 0.5 * sl * (bl - 1)};
                            double v2 = 0.0;
                            for (int x = 0; x < 3; ++x) {
                                const double v = d[0] * recip[x] + d[1] * recip[3 + x] + d[2] * recip[6 + x];
                                v2 += v * v;
                            }
                            rho = fmax(rho, sqrt(v2));
                        }
                const double pass = fmin(1.0, 1.5 * (rho + reach) / fmax(R, 1e-12));
                const double cost = (C0 + (double)O * C1 * pass) / (double)P;
                if (cost < best) {
                    best = cost;
                    best_rho = rho;
                    G.bh = bh; G.bk = bk; G.bl = bl;
                }
            }
    for (int i = 0; i < 3; ++i) G.hmax[i] = hmax[i] > 0 ? hmax[i] : 0;
    G.nbx = (2 * G.hmax[0] + G.bh) / G.bh;
    G.nby = (2 * G.hmax[1] + G.bk) / G.bk;
    G.nbz = (2 * G.hmax[2] + G.bl) / G.bl;
    // margin over the FP32 rounding of the brick and row tests (~1e-6 at
    // |g| of a few 1/Angstrom) and of the band's ends
    G.rho_margin = (float)(best_rho * (1.0 + 1e-5) + 1e-4);
    return G;
}

static inline long long brick_blocks(const BrickGeom &G) { return (long long)G.nbx * G.nby * G.nbz; }
// bricks at most: one per non-empty block plus one per 32 rows
static inline long long brick_max(const BrickGeom &G, long long n_hkl) {
    return std::min(brick_blocks(G), n_hkl) + n_hkl / 32 + 1;
}

size_t brick_scratch_bytes(const BrickGeom &G, long long n_hkl) {
    const long long nblk = brick_blocks(G), nb = brick_max(G, n_hkl);
    size_t o = 0;
    o += align_up((size_t)nblk * 4, 256) * 2;        // counts, fill (zeroed)
    o += align_up(16, 256);                          // meta (zeroed)
    o += align_up((size_t)nblk * 4, 256);            // first brick of each block
    o += align_up((size_t)nb * 4, 256);              // brick -> block
    o += align_up((size_t)nb * 32 * 4, 256);         // slot rows
    o += align_up((size_t)nb * 32 * sizeof(float4), 256);
    o += align_up((size_t)nb * 32 * 4, 256);         // slot z_half
    o += align_up((size_t)nb * sizeof(float4), 256);
    o += align_up((size_t)nb * 4, 256);              // half widths
    return o;
}

ds_status launch_brick_build(const BrickGeom &G, const int32_t *hkl, long long n_hkl, const float4 *scr,
                             const float *zh, void *scratch, TableP &T, cudaStream_t s) {
    const long long nblk = brick_blocks(G), nb = brick_max(G, n_hkl);
    DS_REQUIRE(nblk > 0 && nblk < (1ll << 30) && nb < (1ll << 26), "brick screen: block grid out of range");
    unsigned char *b = reinterpret_cast<unsigned char *>(scratch);
    size_t o = 0;
    int32_t *cnt = reinterpret_cast<int32_t *>(b + o); o += align_up((size_t)nblk * 4, 256);
    int32_t *fill = reinterpret_cast<int32_t *>(b + o); o += align_up((size_t)nblk * 4, 256);
    int32_t *meta = reinterpret_cast<int32_t *>(b + o); o += align_up(16, 256);
    const size_t zero_bytes = o;
    int32_t *first = reinterpret_cast<int32_t *>(b + o); o += align_up((size_t)nblk * 4, 256);
    int32_t *bblk = reinterpret_cast<int32_t *>(b + o); o += align_up((size_t)nb * 4, 256);
    int32_t *bperm = reinterpret_cast<int32_t *>(b + o); o += align_up((size_t)nb * 32 * 4, 256);
    float4 *bscr = reinterpret_cast<float4 *>(b + o); o += align_up((size_t)nb * 32 * sizeof(float4), 256);
    float *bzh = reinterpret_cast<float *>(b + o); o += align_up((size_t)nb * 32 * 4, 256);
    float4 *brec = reinterpret_cast<float4 *>(b + o); o += align_up((size_t)nb * sizeof(float4), 256);
    float *bhalf = reinterpret_cast<float *>(b + o);
    DS_CUDA_TRY(cudaMemsetAsync(b, 0, zero_bytes, s));
    if (n_hkl > 0) {
        const unsigned g = (unsigned)((n_hkl + 255) / 256);
        brick_count_kernel<<<g, 256, 0, s>>>(G, hkl, n_hkl, cnt);
        ds_status st = check_launch("brick_count_kernel");
        if (st) return st;
        brick_scan_kernel<<<1, BRICK_SCAN_THREADS, 0, s>>>((int)nblk, cnt, first, bblk, meta);
        st = check_launch("brick_scan_kernel");
        if (st) return st;
        brick_fill_kernel<<<g, 256, 0, s>>>(G, hkl, n_hkl, first, fill, scr, zh, bperm, bscr, bzh);
        st = check_launch("brick_fill_kernel");
        if (st) return st;
        brick_bounds_kernel<<<(unsigned)((nb * 32 + 255) / 256), 256, 0, s>>>(G, bblk, first, cnt, meta, bperm, bscr,
                                                                           bzh, brec, bhalf);
        st = check_launch("brick_bounds_kernel");
        if (st) return st;
    }
    T.bperm = bperm;
    T.bscr = bscr;
    T.bzh = bzh;
    T.brec = brec;
    T.bhalf = bhalf;
    T.bmeta = meta;
    return DS_OK;
}

constexpr long long STAGE_CAP = 24576;  // staged candidates per pipeline slot (20 bytes each)

struct SimPlan {
    int O, W, Ws;
    long long n_tiles, grid, stage_cap;
    int line_mode, brick_mode;
    long long line_tiles;
    BrickGeom bricks;
    size_t off_lb, off_scr, off_zh, off_g2, off_sidx, off_sI, off_lines, off_lmeta, off_llb, off_bricks, total;
    size_t smem;
};

// Half-thickness of the selection band about the Ewald sphere (1/Angstrom),
// for the brick shape's cost model: s_max, widened by how far the precessing
// sphere strays at the table's largest |g|.
double selection_reach(const ds_sim_params *p, const ds_phase_table *t) {
    double reach = p->max_excitation_error;
    if (p->precession_mode != DS_PRECESSION_NONE) {
        double R = 0.0;
        for (int i = 0; i < 3; ++i)
            R = fmax(R, sqrt(t->recip[3 * i] * t->recip[3 * i] + t->recip[3 * i + 1] * t->recip[3 * i + 1] +
                             t->recip[3 * i + 2] * t->recip[3 * i + 2]) * (double)t->hmax[i]);
        reach += R * sin(p->precession_angle) + p->k0 * (1.0 - cos(p->precession_angle));
    }
    return reach;
}

static int pick_O(const ds_sim_params *p, long long n_hkl, long long n_orient) {
    long long W = (n_hkl + 31) / 32;
    long long Ws = W | 1;
    const int o_cap = p->form == DS_FORM_FP64 ? 16 : SIM_MAX_O;
    if (p->orient_tile > 0) return p->orient_tile < o_cap ? p->orient_tile : o_cap;
    int O = o_cap;
    const long long budget = sim_two_cta_smem();  // two CTAs per SM
    while (O > 1 && (long long)sim_smem_layout(O, (int)Ws).total > budget) O >>= 1;
    // keep at least ~2 tiles per SM when the orientation count allows it
    while (O > 4 && (n_orient + O - 1) / O < 304) O >>= 1;
    return O;
}

static const void *kernel_ptr(int O, int form, bool integ) {
    if (integ) return simulate_kernel_integral(O, form);
    if (form == DS_FORM_FP64) {
        switch (O) {
            case 1: return (const void *)simulate_kernel<1, DS_FORM_FP64, false>;
            case 2: return (const void *)simulate_kernel<2, DS_FORM_FP64, false>;
            case 4: return (const void *)simulate_kernel<4, DS_FORM_FP64, false>;
            case 8: return (const void *)simulate_kernel<8, DS_FORM_FP64, false>;
            default: return (const void *)simulate_kernel<16, DS_FORM_FP64, false>;
        }
    }
    switch (O) {
        case 1: return (const void *)simulate_kernel<1, DS_FORM_MIXED, false>;
        case 2: return (const void *)simulate_kernel<2, DS_FORM_MIXED, false>;
        case 4: return (const void *)simulate_kernel<4, DS_FORM_MIXED, false>;
        case 8: return (const void *)simulate_kernel<8, DS_FORM_MIXED, false>;
        case 16: return (const void *)simulate_kernel<16, DS_FORM_MIXED, false>;
        default: return (const void *)simulate_kernel<32, DS_FORM_MIXED, false>;
    }
}

// Launch plan: tile size, persistent grid (resident CTAs, at most one per
// tile) and the scratch layout.
static ds_status make_plan(const ds_sim_params *p, const ds_phase_table *t, long long n_orient, SimPlan &P) {
    // screen: per-row tests by default; per-(orientation, line) intervals on
    // request for the mixed form without precession (the band of the
    // precessing sphere is not quadratic in l).  With ~30 rows per line the
    // interval arithmetic costs about what the row tests do.
    P.line_mode = (p->form == DS_FORM_MIXED && p->precession_mode == DS_PRECESSION_NONE &&
                   p->screen == DS_SCREEN_LINES && t->n_hkl > 0) ? 1 : 0;
    P.brick_mode = (p->form == DS_FORM_MIXED && !P.line_mode && t->n_hkl > 0 && p->screen == DS_SCREEN_BRICKS) ? 1 : 0;
    P.line_tiles = (t->n_hkl + LN_TILE - 1) / LN_TILE;
    P.O = pick_O(p, t->n_hkl, n_orient);
    if (p->form == DS_FORM_FP64 && P.O > 16) P.O = 16;
    P.W = (int)((t->n_hkl + 31) / 32);
    P.Ws = P.W | 1;
    P.n_tiles = (n_orient + P.O - 1) / P.O;
    P.smem = sim_smem_layout(P.O, P.Ws).total;
    DS_REQUIRE(P.smem <= 227 * 1024, "ds_simulate: candidate table too large for one orientation tile");
    const void *kern = kernel_ptr(P.O, p->form, p->precession_mode == DS_PRECESSION_INTEGRAL);
    DS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem));
    int dev = 0, n_sm = 0, per_sm = 0;
    DS_CUDA_TRY(cudaGetDevice(&dev));
    DS_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    DS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SIM_THREADS, P.smem));
    if (per_sm < 1) per_sm = 1;
    long long resident = (long long)n_sm * per_sm;
    P.grid = P.n_tiles < resident ? P.n_tiles : resident;
    if (P.grid < 1) P.grid = 1;
    long long most = (long long)P.O * t->n_hkl;
    const long long cap = p->stage_cap > 0 ? p->stage_cap : STAGE_CAP;
    P.stage_cap = most < cap ? most : cap;
    if (P.stage_cap < 1) P.stage_cap = 1;
    size_t o = 0;
    P.off_lb = o; o += lookback_scratch_bytes(P.n_tiles);
    o = align_up(o, 256);
    P.off_scr = o; o += (size_t)t->n_hkl * sizeof(float4);
    o = align_up(o, 256);
    P.off_zh = o; o += (size_t)t->n_hkl * sizeof(float);
    o = align_up(o, 256);
    P.off_g2 = o; o += (size_t)t->n_hkl * 2 * sizeof(float4);
    o = align_up(o, 256);
    P.off_sidx = o; o += (size_t)(2 * P.grid * P.stage_cap) * sizeof(int32_t);  // two pipeline slots per CTA
    o = align_up(o, 256);
    P.off_sI = o; o += (size_t)(2 * P.grid * P.stage_cap) * sizeof(float);
    o = align_up(o, 256);
    P.off_lines = o; o += P.line_mode ? (size_t)t->n_hkl * sizeof(LineP) : 0;
    o = align_up(o, 256);
    P.off_lmeta = o; o += 256;
    P.off_llb = o; o += P.line_mode ? lookback_scratch_bytes(P.line_tiles) : 0;
    o = align_up(o, 256);
    P.off_bricks = o;
    if (P.brick_mode) {
        P.bricks = brick_geometry(t->recip, t->hmax, P.O, selection_reach(p, t));
        o += brick_scratch_bytes(P.bricks, t->n_hkl);
    }
    P.total = align_up(o, 256);
    return DS_OK;
}

ds_status launch_sim_prep(const SimConst &c, const int32_t *hkl, const double *g2, const float *F2, float4 *scr, float *zh, float4 *aux,
                          long long n_hkl, cudaStream_t s) {
    if (n_hkl <= 0) return DS_OK;
    sim_prep_kernel<<<(unsigned)((n_hkl + 255) / 256), 256, 0, s>>>(c, hkl, g2, F2, scr, zh, aux);
    return check_launch("sim_prep_kernel");
}

static ds_status launch_sim(const void *kern, SimConst c, TableP T, const double *quats, ds_spots *out,
                            LookbackScratch lb, StageP stg, const SimPlan &P, int32_t *status, cudaStream_t s) {
    int64_t *offsets = out->offsets, *total = out->total;
    int32_t *idx = out->hkl_index;
    float4 *xyzi = reinterpret_cast<float4 *>(out->xyzi);
    double *sv = out->excitation_error;
    void *args[] = {&c, &T, &quats, &offsets, &idx, &xyzi, &sv, &total, &lb, &stg, &status};
    DS_CUDA_TRY(cudaLaunchKernel(kern, dim3((unsigned)P.grid), dim3(SIM_THREADS), args, P.smem, s));
    return check_launch("simulate_kernel");
}

// Scratch of ds_simulate for one problem, with make_plan's own status and
// message on failure: the bytes at the staging capacity of p (or the
// default), the staging capacity the plan uses, and the bytes one more unit
// of staging capacity adds (two slots of (row, I) per CTA).
ds_status simulate_scratch_plan(const ds_sim_params *p, const ds_phase_table *t, long long n_orient,
                                size_t *total, long long *stage_cap, size_t *per_stage) {
    DS_REQUIRE(p && t && total && stage_cap && per_stage, "simulate_scratch_plan: null pointer");
    SimPlan P;
    ds_status st = make_plan(p, t, n_orient, P);
    if (st) return st;
    *total = P.total;
    *stage_cap = P.stage_cap;
    *per_stage = (size_t)(2 * P.grid) * (sizeof(int32_t) + sizeof(float));
    return DS_OK;
}

}  // namespace ds

using namespace ds;

extern "C" size_t ds_simulate_scratch_bytes(const ds_sim_params *p, const ds_phase_table *t, int64_t n_orient) {
    if (!p || !t || n_orient <= 0) return 0;
    SimPlan P;
    if (make_plan(p, t, n_orient, P) != DS_OK) return 0;
    return P.total;
}

extern "C" ds_status ds_simulate(const ds_sim_params *p, const ds_phase_table *t, const double *quats,
                                 int64_t n_orient, ds_spots *out, void *scratch, size_t scratch_bytes,
                                 int32_t *status, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_simulate");
    DS_REQUIRE(p && t && out && status, "ds_simulate: null pointer");
    DS_REQUIRE(n_orient >= 0, "ds_simulate: n_orient < 0");
    DS_REQUIRE(t->n_hkl >= 0 && t->n_hkl < (1ll << 31), "ds_simulate: n_hkl out of range");
    {
        ds_status vs = validate_params(p, "ds_simulate");
        if (vs) return vs;
    }
    DS_REQUIRE(out->hkl_index_bytes == 0 || out->hkl_index_bytes == 4 ||
                   (out->hkl_index_bytes == 2 && t->n_hkl <= 65536),
               "ds_simulate: hkl_index_bytes must be 0 or 4, or 2 for tables of at most 65536 rows");
    cudaStream_t s = (cudaStream_t)stream;
    if (n_orient == 0) {
        DS_CUDA_TRY(cudaMemsetAsync(out->offsets, 0, sizeof(int64_t), s));
        DS_CUDA_TRY(cudaMemsetAsync(out->total, 0, sizeof(int64_t), s));
        return DS_OK;
    }
    DS_REQUIRE(quats && out->offsets && out->total, "ds_simulate: null quats / offsets / total");
    DS_REQUIRE(t->n_hkl == 0 || (t->hkl && t->g2 && (p->form == DS_FORM_MIXED ? t->F2 != nullptr : t->F2d != nullptr)),
               "ds_simulate: table arrays missing for this form");
    DS_REQUIRE(out->capacity >= 0 && (out->capacity == 0 || (out->hkl_index && out->xyzi)),
               "ds_simulate: output arrays missing");
    DS_REQUIRE(((uintptr_t)out->xyzi & 15) == 0, "ds_simulate: xyzi must be 16-byte aligned");
    SimPlan P;
    ds_status pst = make_plan(p, t, n_orient, P);
    if (pst != DS_OK) return pst;
    DS_REQUIRE(scratch && scratch_bytes >= P.total, "ds_simulate: scratch too small");

    SimConst c;
    fill_const(p, t, c);
    c.O = P.O;
    c.W = P.W;
    c.Ws = P.Ws;
    c.n_orient = n_orient;
    c.line_mode = P.line_mode;
    c.parts_log2 = refine_parts_log2(p, P.O);
    c.n_tiles = P.n_tiles;
    c.capacity = out->capacity;
    c.idx16 = out->hkl_index_bytes == 2;

    unsigned char *sb = reinterpret_cast<unsigned char *>(scratch);
    TableP T;
    T.scr = reinterpret_cast<float4 *>(sb + P.off_scr);
    T.zh = reinterpret_cast<float *>(sb + P.off_zh);
    T.aux = reinterpret_cast<float4 *>(sb + P.off_g2);
    T.F2d = t->F2d;
    DS_CUDA_TRY(cudaMemsetAsync(sb + P.off_lb, 0, lookback_scratch_bytes(P.n_tiles), s));
    if (t->n_hkl > 0) {
        sim_prep_kernel<<<(unsigned)((t->n_hkl + 255) / 256), 256, 0, s>>>(
            c, t->hkl, t->g2, p->form == DS_FORM_MIXED ? t->F2 : nullptr, const_cast<float4 *>(T.scr),
            const_cast<float *>(T.zh), const_cast<float4 *>(T.aux));
        ds_status st = check_launch("sim_prep_kernel");
        if (st) return st;
    }
    T.lines = reinterpret_cast<const LineP *>(sb + P.off_lines);
    T.line_meta = reinterpret_cast<const int *>(sb + P.off_lmeta);
    T.bperm = T.bmeta = nullptr;
    T.bscr = T.brec = nullptr;
    T.bzh = T.bhalf = nullptr;
    c.brick_mode = P.brick_mode;
    if (P.brick_mode) {
        ds_status st = launch_brick_build(P.bricks, t->hkl, t->n_hkl, T.scr, T.zh, sb + P.off_bricks, T, s);
        if (st) return st;
    }
    if (P.line_mode) {
        DS_CUDA_TRY(cudaMemsetAsync(sb + P.off_lmeta, 0x7f, 256, s));  // [1] = no 000 row yet (0x7f7f7f7f)
        DS_CUDA_TRY(cudaMemsetAsync(sb + P.off_llb, 0, lookback_scratch_bytes(P.line_tiles), s));
        lines_kernel<<<(unsigned)P.line_tiles, LN_THREADS, 0, s>>>(
            c, t->hkl, reinterpret_cast<LineP *>(sb + P.off_lines), reinterpret_cast<int *>(sb + P.off_lmeta),
            lookback_scratch(sb + P.off_llb), P.line_tiles, status);
        ds_status st = check_launch("lines_kernel");
        if (st) return st;
    }
    LookbackScratch lb = lookback_scratch(sb + P.off_lb);
    StageP stg;
    stg.idx = reinterpret_cast<int32_t *>(sb + P.off_sidx);
    stg.inten = reinterpret_cast<float *>(sb + P.off_sI);
    stg.cap = P.stage_cap;
    return launch_sim(kernel_ptr(P.O, p->form, p->precession_mode == DS_PRECESSION_INTEGRAL), c, T, quats, out, lb,
                      stg, P, status, s);
}
