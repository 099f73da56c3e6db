// Many phases in one persistent launch (no counterpart in the reference, which
// loops over phases and orientations in Python,
// diffsims/generators/simulation_generator.py:198-241): every phase's
// orientations are cut into tiles of O; one tile ticket runs over all tiles,
// phase after phase, so a CTA that finishes a small phase moves straight on to
// the next phase's tiles and the launch has no per-phase tail; the look-back
// orders the output across phases (one CSR, phase-major).  The phases'
// descriptors travel as one kernel parameter (graph-capturable, no host
// buffer to keep alive).
#include <algorithm>

#include "simulate_kernel.cuh"

namespace ds {

const void *simulate_batch_kernel_plain(int O, int form) {
    if (form == DS_FORM_FP64) {
        switch (O) {
            case 1: return (const void *)simulate_batch_kernel<1, DS_FORM_FP64, false>;
            case 2: return (const void *)simulate_batch_kernel<2, DS_FORM_FP64, false>;
            case 4: return (const void *)simulate_batch_kernel<4, DS_FORM_FP64, false>;
            default: return (const void *)simulate_batch_kernel<8, DS_FORM_FP64, false>;
        }
    }
    switch (O) {
        case 1: return (const void *)simulate_batch_kernel<1, DS_FORM_MIXED, false>;
        case 2: return (const void *)simulate_batch_kernel<2, DS_FORM_MIXED, false>;
        case 4: return (const void *)simulate_batch_kernel<4, DS_FORM_MIXED, false>;
        case 8: return (const void *)simulate_batch_kernel<8, DS_FORM_MIXED, false>;
        case 16: return (const void *)simulate_batch_kernel<16, DS_FORM_MIXED, false>;
        default: return (const void *)simulate_batch_kernel<32, DS_FORM_MIXED, false>;
    }
}

static inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr long long BATCH_STAGE_CAP = 24576;

struct BatchPlan {
    int O, Ws_max, grid, brick_mode;
    int Op[SIM_BATCH_MAX];
    long long n_tiles, n_orient, stage_cap;
    size_t smem, off_lb, off_sidx, off_sI, total;
    size_t off_prep[SIM_BATCH_MAX];    // per phase: scr, zh, aux
    size_t off_bricks[SIM_BATCH_MAX];  // per phase: the brick screen's arrays
    BrickGeom bricks[SIM_BATCH_MAX];
};

static ds_status batch_plan(const ds_sim_params *p, const ds_batch_phase *ph, int n, BatchPlan &P) {
    DS_REQUIRE(n >= 1 && n <= SIM_BATCH_MAX, "ds_simulate_batch: n_phases must be 1..96");
    long long max_hkl = 0, n_orient = 0;
    for (int i = 0; i < n; ++i) {
        DS_REQUIRE(ph[i].table.n_hkl >= 0 && ph[i].table.n_hkl < (1ll << 31), "ds_simulate_batch: n_hkl out of range");
        DS_REQUIRE(ph[i].n_orient >= 0, "ds_simulate_batch: n_orient < 0");
        max_hkl = std::max(max_hkl, (long long)ph[i].table.n_hkl);
        n_orient += ph[i].n_orient;
    }
    const int o_cap = p->form == DS_FORM_FP64 ? 8 : (p->precession_mode == DS_PRECESSION_INTEGRAL ? 16 : 32);
    int O = std::min(p->orient_tile > 0 ? (int)p->orient_tile : 16, o_cap);
    O = O >= 32 ? 32 : O >= 16 ? 16 : O >= 8 ? 8 : O >= 4 ? 4 : O >= 2 ? 2 : 1;  // an instantiated tile
    // per phase: the largest tile <= O whose bitmap, with the O-tile's fixed
    // shared data, fits two CTAs per SM; the launch's bitmap holds the
    // largest of them
    const long long budget = sim_two_cta_smem();
    long long words = 1;
    P.n_tiles = 0;
    for (int i = 0; i < n; ++i) {
        const long long Ws = ((ph[i].table.n_hkl + 31) / 32) | 1;
        int Op = O;
        while (Op > 1 && (long long)sim_smem_layout(O, (int)((Op * Ws + O - 1) / O)).total > budget) Op >>= 1;
        P.Op[i] = Op;
        words = std::max(words, (long long)Op * Ws);
        P.n_tiles += (ph[i].n_orient + Op - 1) / Op;
    }
    P.O = O;
    P.Ws_max = (int)((words + O - 1) / O);  // bitmap of O rows of Ws_max words >= every phase's
    P.n_orient = n_orient;
    P.smem = sim_smem_layout(O, P.Ws_max).total;
    DS_REQUIRE(P.smem <= 227 * 1024, "ds_simulate_batch: candidate table too large for one orientation tile");
    const void *kern = p->precession_mode == DS_PRECESSION_INTEGRAL ? simulate_batch_kernel_integral(O, p->form)
                                                                    : simulate_batch_kernel_plain(O, p->form);
    DS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem));
    int dev = 0, n_sm = 0, per_sm = 0;
    DS_CUDA_TRY(cudaGetDevice(&dev));
    DS_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    DS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SIM_THREADS, P.smem));
    if (per_sm < 1) per_sm = 1;
    const long long resident = (long long)n_sm * per_sm;
    P.grid = (int)std::max(1ll, std::min(P.n_tiles, resident));
    const long long cap = p->stage_cap > 0 ? p->stage_cap : BATCH_STAGE_CAP;
    P.stage_cap = std::max(1ll, std::min((long long)O * max_hkl, cap));  // O x rows bounds any tile's candidates
    size_t o = 0;
    P.off_lb = o; o += lookback_scratch_bytes(P.n_tiles);
    for (int i = 0; i < n; ++i) {
        o = align256(o);
        P.off_prep[i] = o;
        const size_t nh = (size_t)ph[i].table.n_hkl;
        o += align256(nh * sizeof(float4)) + align256(nh * sizeof(float)) + align256(nh * 2 * sizeof(float4));
    }
    P.brick_mode = (p->form == DS_FORM_MIXED && p->screen == DS_SCREEN_BRICKS) ? 1 : 0;
    for (int i = 0; i < n; ++i) {
        o = align256(o);
        P.off_bricks[i] = o;
        if (P.brick_mode && ph[i].table.n_hkl > 0) {
            P.bricks[i] = brick_geometry(ph[i].table.recip, ph[i].table.hmax, P.Op[i], selection_reach(p, &ph[i].table));
            o += brick_scratch_bytes(P.bricks[i], ph[i].table.n_hkl);
        }
    }
    o = align256(o);
    P.off_sidx = o; o += (size_t)(2 * P.grid * P.stage_cap) * sizeof(int32_t);
    o = align256(o);
    P.off_sI = o; o += (size_t)(2 * P.grid * P.stage_cap) * sizeof(float);
    P.total = align256(o);
    return DS_OK;
}

}  // namespace ds

using namespace ds;

extern "C" size_t ds_simulate_batch_scratch_bytes(const ds_sim_params *p, const ds_batch_phase *phases,
                                                  int32_t n_phases) {
    clear_error();
    if (!p || !phases || n_phases < 1) return 0;
    BatchPlan P;
    if (batch_plan(p, phases, n_phases, P) != DS_OK) return 0;
    return P.total;
}

extern "C" int32_t ds_simulate_batch_tile(const ds_sim_params *p, const ds_batch_phase *phases, int32_t n_phases) {
    clear_error();
    if (!p || !phases || n_phases < 1) return 0;
    BatchPlan P;
    if (batch_plan(p, phases, n_phases, P) != DS_OK) return 0;
    return P.O;
}

extern "C" ds_status ds_simulate_batch(const ds_sim_params *p, const ds_batch_phase *phases, int32_t n_phases,
                                       ds_spots *out, void *scratch, size_t scratch_bytes, int32_t *status,
                                       void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_simulate_batch");
    DS_REQUIRE(p && phases && out && status, "ds_simulate_batch: null pointer");
    {
        ds_status vs = validate_params(p, "ds_simulate_batch");
        if (vs) return vs;
    }
    DS_REQUIRE(out->hkl_index_bytes == 0 || out->hkl_index_bytes == 4,
               "ds_simulate_batch: hkl_index_bytes must be 0 or 4 (int32 rows)");
    DS_REQUIRE(p->orient_tile == 0 || p->orient_tile <= (p->form == DS_FORM_FP64 ? 8 : 32),
               "ds_simulate_batch: orient_tile must be <= 32 (mixed; 16 with the precession average) or 8 (FP64)");
    BatchPlan P;
    ds_status st = batch_plan(p, phases, n_phases, P);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    DS_REQUIRE(out->offsets && out->total, "ds_simulate_batch: null offsets / total");
    if (P.n_orient == 0) {
        DS_CUDA_TRY(cudaMemsetAsync(out->offsets, 0, sizeof(int64_t), s));
        DS_CUDA_TRY(cudaMemsetAsync(out->total, 0, sizeof(int64_t), s));
        return DS_OK;
    }
    DS_REQUIRE(out->capacity >= 0 && (out->capacity == 0 || (out->hkl_index && out->xyzi)),
               "ds_simulate_batch: output arrays missing");
    DS_REQUIRE(((uintptr_t)out->xyzi & 15) == 0, "ds_simulate_batch: xyzi must be 16-byte aligned");
    DS_REQUIRE(scratch && scratch_bytes >= P.total, "ds_simulate_batch: scratch too small");
    unsigned char *sb = reinterpret_cast<unsigned char *>(scratch);

    // launch-wide constants from the first phase; every phase's own below
    SimConst c;
    fill_const(p, &phases[0].table, c);
    c.O = P.O;
    c.Ws = P.Ws_max;
    c.n_orient = P.n_orient;
    c.n_tiles = P.n_tiles;
    c.capacity = out->capacity;
    c.line_mode = 0;
    c.brick_mode = P.brick_mode;
    c.parts_log2 = refine_parts_log2(p, P.O);

    PhaseBatch B;
    B.n = n_phases;
    long long tile0 = 0, orient0 = 0;
    for (int i = 0; i < n_phases; ++i) {
        const ds_phase_table *t = &phases[i].table;
        const long long nh = t->n_hkl, no = phases[i].n_orient;
        DS_REQUIRE(no == 0 || phases[i].quats, "ds_simulate_batch: null quats");
        DS_REQUIRE(nh == 0 || (t->hkl && t->g2 && (p->form == DS_FORM_MIXED ? t->F2 != nullptr : t->F2d != nullptr)),
                   "ds_simulate_batch: table arrays missing for this form");
        SimConst cp;
        fill_const(p, t, cp);
        PhaseP &d = B.ph[i];
        unsigned char *base = sb + P.off_prep[i];
        float4 *scr = reinterpret_cast<float4 *>(base);
        float *zh = reinterpret_cast<float *>(base + align256(nh * sizeof(float4)));
        float4 *aux = reinterpret_cast<float4 *>(base + align256(nh * sizeof(float4)) + align256(nh * sizeof(float)));
        d.T.scr = scr;
        d.T.zh = zh;
        d.T.aux = aux;
        d.T.F2d = t->F2d;
        d.T.lines = nullptr;
        d.T.line_meta = nullptr;
        d.T.bperm = d.T.bmeta = nullptr;
        d.T.bscr = d.T.brec = nullptr;
        d.T.bzh = d.T.bhalf = nullptr;
        d.quats = phases[i].quats;
        for (int k = 0; k < 9; ++k) d.recip[k] = cp.recip[k];
        for (int k = 0; k < 3; ++k) d.hmax[k] = cp.hmax[k];
        d.W = cp.W;
        d.Ws = cp.Ws;
        d.n_hkl = nh;
        d.n_orient = no;
        d.O = P.Op[i];
        d.tile0 = tile0;
        d.n_tiles = (no + d.O - 1) / d.O;
        d.orient0 = orient0;
        tile0 += d.n_tiles;
        orient0 += no;
        st = launch_sim_prep(cp, t->hkl, t->g2, p->form == DS_FORM_MIXED ? t->F2 : nullptr, scr, zh, aux, nh, s);
        if (st) return st;
        if (P.brick_mode && nh > 0) {
            st = launch_brick_build(P.bricks[i], t->hkl, nh, scr, zh, sb + P.off_bricks[i], d.T, s);
            if (st) return st;
        }
    }
    DS_CUDA_TRY(cudaMemsetAsync(sb + P.off_lb, 0, lookback_scratch_bytes(P.n_tiles), s));
    LookbackScratch lb = lookback_scratch(sb + P.off_lb);
    StageP stg;
    stg.idx = reinterpret_cast<int32_t *>(sb + P.off_sidx);
    stg.inten = reinterpret_cast<float *>(sb + P.off_sI);
    stg.cap = P.stage_cap;
    const void *kern = p->precession_mode == DS_PRECESSION_INTEGRAL ? simulate_batch_kernel_integral(P.O, p->form)
                                                                    : simulate_batch_kernel_plain(P.O, p->form);
    int64_t *offsets = out->offsets, *total = out->total;
    int32_t *idx = out->hkl_index;
    float4 *xyzi = reinterpret_cast<float4 *>(out->xyzi);
    double *sv = out->excitation_error;
    void *args[] = {&c, &B, &offsets, &idx, &xyzi, &sv, &total, &lb, &stg, &status};
    DS_CUDA_TRY(cudaLaunchKernel(kern, dim3((unsigned)P.grid), dim3(SIM_THREADS), args, P.smem, s));
    return check_launch("simulate_batch_kernel");
}
