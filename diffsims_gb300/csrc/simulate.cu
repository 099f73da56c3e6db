// A4-A7 host side: launch plan, scratch layout and the ds_simulate entry
// point of the orientation kernel (device code in simulate_kernel.cuh).
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
                                float4 *__restrict__ scr, float *__restrict__ zh, float2 *__restrict__ g2dd) {
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
    scr[j] = make_float4((float)hkl[3 * j], (float)hkl[3 * j + 1], (float)hkl[3 * j + 2], (float)(-zmid));
    zh[j] = (float)zhalf + c.guard;
    float hi, lo;
    split_double(gsq, hi, lo);
    g2dd[j] = make_float2(hi, lo);
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

constexpr long long STAGE_CAP = 24576;  // staged candidates per pipeline slot (20 bytes each)

struct SimPlan {
    int O, W, Ws;
    long long n_tiles, grid, stage_cap;
    int line_mode;
    long long line_tiles;
    size_t off_lb, off_scr, off_zh, off_g2, off_sidx, off_sI, off_lines, off_lmeta, off_llb, total;
    size_t smem;
};

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
    P.off_g2 = o; o += (size_t)t->n_hkl * sizeof(float2);
    o = align_up(o, 256);
    P.off_sidx = o; o += (size_t)(2 * P.grid * P.stage_cap) * sizeof(int32_t);  // two pipeline slots per CTA
    o = align_up(o, 256);
    P.off_sI = o; o += (size_t)(2 * P.grid * P.stage_cap) * sizeof(float);
    o = align_up(o, 256);
    P.off_lines = o; o += P.line_mode ? (size_t)t->n_hkl * sizeof(LineP) : 0;
    o = align_up(o, 256);
    P.off_lmeta = o; o += 256;
    P.off_llb = o; o += P.line_mode ? lookback_scratch_bytes(P.line_tiles) : 0;
    P.total = align_up(o, 256);
    return DS_OK;
}

ds_status launch_sim_prep(const SimConst &c, const int32_t *hkl, const double *g2, float4 *scr, float *zh, float2 *g2dd,
                          long long n_hkl, cudaStream_t s) {
    if (n_hkl <= 0) return DS_OK;
    sim_prep_kernel<<<(unsigned)((n_hkl + 255) / 256), 256, 0, s>>>(c, hkl, g2, scr, zh, g2dd);
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
    DS_REQUIRE(p && t && out && status, "ds_simulate: null pointer");
    DS_REQUIRE(n_orient >= 0, "ds_simulate: n_orient < 0");
    DS_REQUIRE(t->n_hkl >= 0 && t->n_hkl < (1ll << 31), "ds_simulate: n_hkl out of range");
    {
        ds_status vs = validate_params(p, "ds_simulate");
        if (vs) return vs;
    }
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
    c.n_tiles = P.n_tiles;
    c.capacity = out->capacity;

    unsigned char *sb = reinterpret_cast<unsigned char *>(scratch);
    TableP T;
    T.scr = reinterpret_cast<float4 *>(sb + P.off_scr);
    T.zh = reinterpret_cast<float *>(sb + P.off_zh);
    T.g2dd = reinterpret_cast<float2 *>(sb + P.off_g2);
    T.F2 = t->F2;
    T.F2d = t->F2d;
    DS_CUDA_TRY(cudaMemsetAsync(sb + P.off_lb, 0, lookback_scratch_bytes(P.n_tiles), s));
    if (t->n_hkl > 0) {
        sim_prep_kernel<<<(unsigned)((t->n_hkl + 255) / 256), 256, 0, s>>>(
            c, t->hkl, t->g2, const_cast<float4 *>(T.scr), const_cast<float *>(T.zh), const_cast<float2 *>(T.g2dd));
        ds_status st = check_launch("sim_prep_kernel");
        if (st) return st;
    }
    T.lines = reinterpret_cast<const LineP *>(sb + P.off_lines);
    T.line_meta = reinterpret_cast<const int *>(sb + P.off_lmeta);
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
