// A4-A7: per-orientation spot patterns of one phase (device code; the host
// plan and the C entry point are in simulate.cu).
//
// Replaces the orientation loop of SimulationGenerator.calculate_diffraction2d
// (diffsims/generators/simulation_generator.py:211-241) and
// get_intersecting_reflections (:319-412): rotation of the candidate table
// into the beam frame (R(q)^T g, diffsims/crystallography/_diffracting_vector.py:160),
// excitation error s = k0 - sqrt(k0^2 - r^2) - z, selection (|s| < s_max, or
// the precession band), the rel-rod shape factor, I = sf |F|^2
// (diffsims/utils/sim_utils.py:353), the mask I > max(I) * minimum_intensity
// (:237-240) and ordered compaction of the survivors into CSR.
//
// One CTA owns a tile of O orientations and streams the whole candidate table
// once for all of them:
//   phase 1  FP32 screen.  z = m . hkl (m = R^T-column of the reciprocal basis)
//            against the exact |s| < s_max interval of z for that |g|
//            (precomputed per row) widened by a rounding guard.  One ballot per
//            (32 rows, orientation) writes a word of a shared-memory bitmap.
//   phase 2  refine every screened candidate: double-float (FP32 pair) z, r^2
//            and s; FP64 only when s lies within 1e-9 of the cutoff (FP64
//            step #2); shape factor, intensity, per-orientation max; rejected
//            bits are cleared.  A mask pass runs only if some intensity is
//            positive but <= max * minimum_intensity.
//   phase 3  per-orientation counts, the tile's output offset by decoupled
//            look-back on the tile ticket, then ordered, coalesced writes of
//            (row index) and (x, y, z, I) records.
// The plain all-FP64 form (FORM_FP64) shares phases 2-3 and evaluates every
// (orientation, row) pair in FP64 in phase 1.
#pragma once
#include <math.h>

#include <cmath>
#include <string>
#include <type_traits>

#include "common.cuh"
#include "shape.cuh"

namespace ds {

constexpr int SIM_THREADS = 256;
constexpr int SIM_WARPS = SIM_THREADS / 32;
constexpr float SIM_TAU = 1e-9f;       // | |s| - s_max | below this -> FP64 decision
constexpr float SIM_TAU_SF = 1e-6f;    // |s| this close to a zero of the shape factor -> FP64 s
constexpr float SIM_TAU_PREC = 2e-7f;  // precession band margin below this -> FP64 decision
constexpr float SIM_U_MAX = 0.01f;     // (r / k0)^2 above this -> FP64 (series not used)
constexpr int SIM_MAX_O = 32;
// tuning knob (compile time): chunks screened per step in phase 1
#ifndef DS_SIM_SCREEN_CHUNKS
#define DS_SIM_SCREEN_CHUNKS 2
#endif

struct SimConst {
    double k0, eps, width, phi, thr, Pz, Pt, minima;
    double recip[9];
    dd eps_dd, c2k0_dd, width_dd, mw_dd, phi_dd;
    float k0f, inv_k0sq, eps_f, width_f, sigma_f, mfac_f, phi_f, Pz_f, Pt_f, k0sq_f, guard;
    int shape, prec, form, O;
    int W, Ws;
    int hmax[3];
    int line_mode;                  // phase 1 by per-(orientation, line) intervals
    int brick_mode;                 // phase 1 by bricks (then rows of passing bricks)
    double alpha0, alpha1, beta0, beta1, csq;  // z_a = alpha0 + alpha1 g^2, z_b = beta0 + beta1 g^2, |c*|^2
    float a2f, b2f;                 // -alpha1 |c*|^2, -beta1 |c*|^2
    float inv_a2f, inv_b2f;
    double int_step;                // precession average: breakpoint spacing in s (0: none)
    float int_step_f, mw_f;
    float int_tau;                  // precession average: FP32 result below this -> FP64
    int mask_on, zero_drop;         // thr > 0, thr >= 0 (the FP64 compares done once, on the host)
    int parts_log2;                 // refine / write units: 2^parts_log2 word ranges per orientation (<= 8)
    int idx16;                      // rows written as uint16 (tables of at most 65536 rows)
    float thr_up;                   // >= thr, with margin: FP32 pre-check of I <= max * thr
    long long n_hkl, n_orient, n_tiles, capacity;
};

struct __align__(16) OrientP {
    float4 mz;       // m[2][0..2], 0: the screen's row, one 16-byte shared load
    float m[3][3];   // beam-frame coordinate c = sum_i m[c][i] * hkl_i   (FP32)
    float za[3];     // z column split: za on a power-of-two grid coarse enough that
    float zb[3];     //   sum_i za_i hkl_i is exact in FP32; zb = m - za (small)
    float _pad;
    double M[3][3];  // FP64 copy
};

// per-orientation accumulators in shared memory (ACC_WORDS words each): max I,
// min positive I, count, output offset, then per warp part (up to 8 parts):
// kept count, staging base, candidate count
enum { ACC_MAXI = 0, ACC_MINPOS = 1, ACC_CNT = 2, ACC_OFF = 3, ACC_PART0 = 4, ACC_CBASE0 = 12, ACC_CCNT0 = 20,
       ACC_WORDS = 28 };
// one accumulator block = O orientation slots + 8 words (word 0: tile total)
__host__ __device__ constexpr int acc_stride(int O) { return O * ACC_WORDS + 8; }

struct SimSmem {
    size_t orient, bitmap, acc, queue, total;
};
constexpr int SIM_QCAP = 128;  // per-warp candidate queue (shared memory)
__host__ __device__ inline SimSmem sim_smem_layout(int O, int Ws) {
    SimSmem L;
    size_t o = 0;
    L.orient = o; o += (size_t)2 * O * sizeof(OrientP);  // two pipeline buffers
    L.acc = o; o += (size_t)2 * acc_stride(O) * sizeof(unsigned long long);
    L.queue = o; o += (size_t)SIM_WARPS * SIM_QCAP * sizeof(int32_t);
    o = (o + 15) & ~(size_t)15;
    L.bitmap = o; o += (((size_t)O * Ws + 3) & ~(size_t)3) * sizeof(uint32_t);  // whole uint4s (zeroing)
    L.total = o;
    return L;
}


// ------------------------------------------------------------ hkl lines ----
// Rows come in descending (h, k, l) order, so rows sharing (h, k) form a run
// of consecutive l values (|g|^2 is convex in l: the d-spacing filter keeps a
// contiguous range; only (0, 0) has a hole, at the excluded 000) -- a "line".  Along a line z = A + m_z l and
// |g|^2 = P + 2 Q l + C l^2 (A = m_x h + m_y k, P = |h a* + k b*|^2,
// Q = (h a* + k b*).c*, C = |c*|^2), so the screen z_a - G < z < z_b + G
// becomes two quadratic inequalities in l whose roots bound the candidate
// rows of the line: a few per (orientation, line) instead of a test per row.
struct LineP {
    float h, k;           // line indices
    float pa, qa;         // alpha0 - G + alpha1 P, 2 alpha1 Q
    float pb, qb;         // beta0 + G + beta1 P, 2 beta1 Q
    int row0, n, l_top;   // first row, rows, l of the first row (l descends along the line)
    float kc, kq, lmax;   // |pa| + |pb|, |qa| + |qb|, max |l| (error bounds)
};

constexpr int LN_THREADS = 256;
constexpr int LN_ITEMS = 4;
constexpr int LN_TILE = LN_THREADS * LN_ITEMS;

__device__ __forceinline__ bool row_is_zero(const int32_t *hkl, long long j) {
    return hkl[3 * j] == 0 && hkl[3 * j + 1] == 0 && hkl[3 * j + 2] == 0;
}



// Set bits [j1, j2] of one bitmap row (shared memory).
__device__ __forceinline__ void set_bit_range(uint32_t *row, int j1, int j2) {
    const int wa = j1 >> 5, wb = j2 >> 5;
    for (int w = wa; w <= wb; ++w) {
        const int lo = w == wa ? (j1 & 31) : 0;
        const int hi = w == wb ? (j2 & 31) : 31;
        const uint32_t m = (hi == 31 ? 0xFFFFFFFFu : ((1u << (hi + 1)) - 1u)) & ~((1u << lo) - 1u);
        atomicOr(&row[w], m);
    }
}

// Candidate rows of one (orientation, line): the l where
//   qa(l) = a2 l^2 + (m_z - qa) l + (A - pa) > 0    (z > z_a - G; a2 < 0: between roots)
//   qb(l) = b2 l^2 + (m_z - qb) l + (A - pb) < 0    (z < z_b + G; b2 < 0: outside roots)
// Roots by the stable quadratic formula with fast reciprocal / square-root
// approximations (a few ulp); every root is pushed outward (the kept set only
// grows) by a bound on its FP32 error plus 1e-3 of a row, so the rows marked
// are a superset of the rows the exact screen keeps.
__device__ __forceinline__ void line_candidates(const SimConst &c, const LineP &L, float mx, float my, float mz,
                                                uint32_t *row) {
    const float A = fmaf(mx, L.h, my * L.k);
    const float ca1 = mz - L.qa, ca0 = A - L.pa;
    const float cb1 = mz - L.qb, cb0 = A - L.pb;
    // FP32 error bound of the coefficients (L.kc = |pa| + |pb|, L.kq = |qa| + |qb|, L.lmax = max |l|)
    const float dc = 8.f * 5.96e-8f * (fabsf(mx * L.h) + fabsf(my * L.k) + L.kc + (fabsf(mz) + L.kq) * L.lmax) + 1e-12f;
    const float fa = -4.f * c.a2f * ca0;
    const float Da = fmaf(ca1, ca1, fa) + 1e-5f * (ca1 * ca1 + fabsf(fa)) + 4.f * fabsf(c.a2f) * dc;
    if (!(Da > 0.f)) return;  // qa <= 0 on the whole line
    const float ia = rsqrtf(Da);
    const float sa = Da * ia;
    const float ta = -0.5f * (ca1 + copysignf(sa, ca1));
    const float r1 = __fdividef(ca0, ta), r2 = ta * c.inv_a2f;
    const float ma = 2.f * dc * ia + 1e-3f + 1e-5f * (fabsf(r1) + fabsf(r2));
    const float a_lo = fminf(r1, r2) - ma, a_hi = fmaxf(r1, r2) + ma;
    const float fb = -4.f * c.b2f * cb0;
    const float Db = fmaf(cb1, cb1, fb) - 1e-5f * (cb1 * cb1 + fabsf(fb)) - 4.f * fabsf(c.b2f) * dc;
    float b_lo = INFINITY, b_hi = -INFINITY;  // excluded open interval (b_lo, b_hi)
    if (Db > 0.f) {
        const float ib = rsqrtf(Db);
        const float sb = Db * ib;
        const float tb = -0.5f * (cb1 + copysignf(sb, cb1));
        const float s1 = __fdividef(cb0, tb), s2 = tb * c.inv_b2f;
        const float mb = 2.f * dc * ib + 1e-3f + 1e-5f * (fabsf(s1) + fabsf(s2));
        b_lo = fminf(s1, s2) + mb;
        b_hi = fmaxf(s1, s2) - mb;
    }
    const float l_bot = (float)(L.l_top - L.n + 1), l_top = (float)L.l_top;
    const bool split = b_lo < b_hi;
    // first interval (a_lo, min(a_hi, b_lo)); second (max(a_lo, b_hi), a_hi) when B excludes a middle part
    const float x2a = split ? fminf(a_hi, b_lo) : a_hi;
    float flo = fmaxf(ceilf(a_lo), l_bot), fhi = fminf(floorf(x2a), l_top);
    if (flo <= fhi) set_bit_range(row, L.row0 + (L.l_top - (int)fhi), L.row0 + (L.l_top - (int)flo));
    if (split) {
        flo = fmaxf(ceilf(fmaxf(a_lo, b_hi)), l_bot);
        fhi = fminf(floorf(a_hi), l_top);
        if (flo <= fhi) set_bit_range(row, L.row0 + (L.l_top - (int)fhi), L.row0 + (L.l_top - (int)flo));
    }
}

// --------------------------------------------------------- evaluation ----
// FP64 excitation error and selection in the reference's operation order
// (simulation_generator.py:355-375): FP64 step #2.
__device__ inline bool select_fp64(const SimConst &c, const OrientP &op, double h, double k, double l, double &s,
                                   double &r, double &z) {
    double x = op.M[0][0] * h + op.M[0][1] * k + op.M[0][2] * l;
    double y = op.M[1][0] * h + op.M[1][1] * k + op.M[1][2] * l;
    z = op.M[2][0] * h + op.M[2][1] * k + op.M[2][2] * l;
    r = sqrt(x * x + y * y);
    double zs = -sqrt(c.k0 * c.k0 - r * r) + c.k0;
    s = zs - z;
    if (c.prec == DS_PRECESSION_NONE) return fabs(s) < c.eps;
    double zup = c.Pz - sqrt(c.k0 * c.k0 - (r + c.Pt) * (r + c.Pt));
    double zdo = c.Pz - sqrt(c.k0 * c.k0 - (r - c.Pt) * (r - c.Pt));
    return (z - c.eps <= zup) && (z + c.eps >= zdo);
}

// Mixed-form selection.  s and r returned for the shape factor.
//  z     = Sa + Sb: Sa = za . hkl is exact in FP32 (za on a coarse power-of-two
//          grid), Sb = zb . hkl is a ~2^-16 relative correction: z to ~1e-12.
//  r^2   = g^2 - z^2 as an FP32 pair (no cancellation: z^2 << g^2 near the sphere).
//  w     = k0 - sqrt(k0^2 - r^2) = (r^2 / 2k0)(1 + u/4 + u^2/8 + 5u^3/64 + ...),
//          u = r^2/k0^2 <= 0.01 (series error < 1e-14 relative).
//  s     = w - z as an FP32 pair, error < ~5e-11.  Pairs within 1e-9 of the
//          cutoff are decided in FP64 (FP64 step #2).
__device__ inline bool select_mixed(const SimConst &c, const OrientP &op, const float4 &e, float2 g2p, dd &s,
                                    float &r, dd &r2o, float &zf) {
    const float Sa = fmaf(op.za[0], e.x, fmaf(op.za[1], e.y, op.za[2] * e.z));
    const float Sb = fmaf(op.zb[0], e.x, fmaf(op.zb[1], e.y, op.zb[2] * e.z));
    const float zz = fmaf(Sa, Sa, (2.f * Sa + Sb) * Sb);
    dd r2 = two_sum(g2p.x, -zz);
    r2.lo += g2p.y;
    const float u = r2.hi * c.inv_k0sq;
    bool fallback = u > SIM_U_MAX;
    bool sel = false;
    r = 0.f;
    if (c.prec != DS_PRECESSION_NONE) r = sqrtf(fmaxf(r2.hi, 0.f));
    r2o = r2;
    if (!fallback) {
        const float corr = u * (0.25f + u * (0.125f + u * (0.078125f + u * (0.0546875f + u * 0.041015625f))));
        const float w0h = r2.hi * c.c2k0_dd.hi;
        const float w0l = fmaf(r2.hi, c.c2k0_dd.hi, -w0h) + fmaf(r2.hi, c.c2k0_dd.lo, r2.lo * c.c2k0_dd.hi);
        const dd t = two_sum(w0h, -Sa);
        s = two_sum(t.hi, t.lo + (w0l - Sb) + w0h * corr);
        if (c.prec == DS_PRECESSION_NONE) {
            // |s| - eps: the leading difference is exact (Sterbenz) whenever it matters
            const float sg = s.hi < 0.f ? -1.f : 1.f;
            const float d = (fabsf(s.hi) - c.eps_dd.hi) + (sg * s.lo - c.eps_dd.lo);
            if (fabsf(d) < SIM_TAU) fallback = true;
            else sel = d < 0.f;
            // near a zero of the shape factor the intensity's relative error is
            // that of |s| - s_zero: take s from FP64 there too
            if (sel && !fallback) {
                if (c.shape == DS_SHAPE_LINEAR) {
                    const float dz = (fabsf(s.hi) - c.width_dd.hi) + (sg * s.lo - c.width_dd.lo);
                    if (fabsf(dz) < SIM_TAU_SF) fallback = true;
                } else if (c.shape == DS_SHAPE_SINC || c.shape == DS_SHAPE_SIN2C) {
                    const float x = fabsf(s.hi + s.lo) * c.mw_dd.hi;  // |s| m / w
                    const float n = rintf(x);
                    if (n >= 1.f && fabsf(x - n) < SIM_TAU_SF * c.mw_dd.hi) fallback = true;
                }
            }
        } else {
            const float zs = Sa + Sb;
            const float rp = r + c.Pt_f, rm = r - c.Pt_f;
            const float a1 = c.k0sq_f - rp * rp, a2 = c.k0sq_f - rm * rm;
            if (!(a1 > 0.f) || !(a2 > 0.f)) {
                fallback = true;
            } else {
                const float zup = r * (r + 2.f * c.Pt_f) / (c.Pz_f + sqrtf(a1));
                const float zdo = r * (r - 2.f * c.Pt_f) / (c.Pz_f + sqrtf(a2));
                const float d1 = zup - (zs - c.eps_f), d2 = (zs + c.eps_f) - zdo;
                if (fabsf(d1) < SIM_TAU_PREC || fabsf(d2) < SIM_TAU_PREC) fallback = true;
                else sel = (d1 >= 0.f) && (d2 >= 0.f);
            }
        }
    }
    if (fallback) {
        double s64, r64, z64;
        sel = select_fp64(c, op, (double)e.x, (double)e.y, (double)e.z, s64, r64, z64);
        split_double(s64, s.hi, s.lo);
        r = (float)r64;
        split_double(r64 * r64, r2o.hi, r2o.lo);
        zf = (float)z64;
        return sel;
    }
    zf = Sa + Sb;
    return sel;
}

// The linear model's rotation average in FP32 pairs, the closed form of
// linear_precession_closed (shape.cuh) restated so that no step subtracts
// nearly equal numbers: every sine and cosine comes from the exactly summed
// distances dt = (s0 + a) - b and db = b - (s0 - a) of a breakpoint b
// (+w, 0, -w) to the ends of [s0 - a, s0 + a] -- sin(t/2) = sqrt(dt / 2a),
// cos(t/2) = sqrt(db / 2a), cos t = (b - s0) / a --, a piece's half-length
// from sin(D/2) = (b_A - b_B) / (2a (S_B C_A + C_B S_A)) and cos(D/2) =
// C_A C_B + S_A S_B, and each of [0, w] and [-w, 0] is integrated about its
// end of smaller shape factor f_E:
//   f_E D + (a/w) [sin t_E (1 - cos D) +/- cos t_E (D - sin D)],
// whose terms are non-negative or at most a third of the others.  Relative
// error <= 7.4e-7 for averages from 1e-10 to 1 (float32 emulation against
// 50-digit arithmetic, grazing and kink cases included).
__device__ __forceinline__ float d_minus_sin_f(float d) {  // alternating Taylor series, D in [0, pi]
    const float d2 = d * d;
    float acc = 1.f / 121645100408832000.f;
    acc = 1.f / 355687428096000.f - d2 * acc;
    acc = 1.f / 1307674368000.f - d2 * acc;
    acc = 1.f / 6227020800.f - d2 * acc;
    acc = 1.f / 39916800.f - d2 * acc;
    acc = 1.f / 362880.f - d2 * acc;
    acc = 1.f / 5040.f - d2 * acc;
    acc = 1.f / 120.f - d2 * acc;
    acc = 1.f / 6.f - d2 * acc;
    return d * d2 * acc;
}

struct PrecBreak {
    float S, C;  // sin(t/2), cos(t/2)
    dd pos;      // s at the angle (the breakpoint, or the range end it is clamped to)
};

__device__ inline float linear_precession_closed_f32(dd s0, dd a, dd w) {
    const float af = a.hi + a.lo, wf = w.hi + w.lo, two_a = 2.f * af, ra = af / wf;
    const dd P = dd_add(s0, a), Q = dd_sub(s0, a);
    auto brk = [&](dd b) {
        PrecBreak X;
        const dd t = dd_sub(P, b), u = dd_sub(b, Q);
        const float dt = t.hi + t.lo, db = u.hi + u.lo;
        if (!(dt > 0.f)) {
            X.S = 0.f; X.C = 1.f; X.pos = P;   // t = 0
        } else if (!(db > 0.f)) {
            X.S = 1.f; X.C = 0.f; X.pos = Q;   // t = pi
        } else {
            X.S = sqrtf(dt / two_a); X.C = sqrtf(db / two_a); X.pos = b;
        }
        return X;
    };
    auto piece = [&](const PrecBreak &A, const PrecBreak &B, float &h) {  // D = t_B - t_A
        const dd nb = dd_sub(A.pos, B.pos);
        const float den = B.S * A.C + B.C * A.S;
        h = den > 0.f ? (nb.hi + nb.lo) / (two_a * den) : 0.f;
        return 2.f * atan2f(h, B.C * A.C + B.S * A.S);
    };
    const dd zero = {0.f, 0.f};
    const PrecBreak Tw = brk(w), T0 = brk(zero), Tm = brk(dd_neg(w));
    float tot = 0.f, h;
    float d = piece(Tw, T0, h);  // [0, w]: f = (w - s) / w, about its start
    if (d > 0.f) {
        const dd fe = dd_sub(w, Tw.pos), ce = dd_sub(Tw.pos, s0);
        tot += (fe.hi + fe.lo) / wf * d +
               ra * (2.f * Tw.S * Tw.C * (2.f * h * h) + (ce.hi + ce.lo) / af * d_minus_sin_f(d));
    }
    d = piece(T0, Tm, h);  // [-w, 0]: f = (w + s) / w, about its end
    if (d > 0.f) {
        const dd fe = dd_add(w, Tm.pos), ce = dd_sub(Tm.pos, s0);
        tot += (fe.hi + fe.lo) / wf * d +
               ra * (2.f * Tm.S * Tm.C * (2.f * h * h) - (ce.hi + ce.lo) / af * d_minus_sin_f(d));
    }
    return tot / 3.14159265358979f;
}

// shape factors, mixed form (diffsims/utils/shape_factor_models.py)
template <bool INTEG>
__device__ inline float shape_mixed(const SimConst &c, dd s, float r, dd r2) {
    if (c.prec == DS_PRECESSION_LORENTZIAN) {  // lorentzian_precession, :183-219
        float sf = s.hi + s.lo;
        float rphi = r * c.phi_f, as = fabsf(sf);
        float A = (rphi - as) * (rphi + as);            // r^2 phi^2 - s^2 without cancellation
        float sig = c.sigma_f;
        float u = fmaf(sig * sig, A, 1.f);
        float q = 2.f * sig * sf;
        float z = sqrtf(fmaf(u, u, q * q));
        float upz = u >= 0.f ? u + z : (q * q) / (z - u);  // u + z, stable for u < 0
        return (sig / 3.14159265358979f) * sqrtf(2.f * upz) / z;
    }
    if (INTEG) {  // _shape_factor_precession, :222-268 (its own kernel instantiation)
        float v;
        bool exact_zero = false;
        if (c.shape == DS_SHAPE_LINEAR && c.width_dd.hi > 0.f) {
            // closed form; r and a = r phi as FP32 pairs from r^2.  A zero
            // from it is exact (the swept range misses the support): no redo
            const float rh = sqrtf(fmaxf(r2.hi, 0.f));
            const dd rr = rh > 0.f ? quick_two_sum(rh, (fmaf(-rh, rh, r2.hi) + r2.lo) / (2.f * rh)) : dd{0.f, 0.f};
            const dd aa = dd_mul(rr, c.phi_dd);
            if (aa.hi > 0.f) {
                v = fmaxf(linear_precession_closed_f32(s, aa, c.width_dd), 0.f);
                exact_zero = v == 0.f;
            } else {
                v = precession_average<float, false>(c, s.hi, s.lo, 0.f, nullptr, nullptr);
            }
        } else {
            v = precession_average<float, false>(c, s.hi, s.lo, r * c.phi_f, nullptr, nullptr);
        }
        if (v < c.int_tau && !exact_zero) {
            // small averages carry the FP32 rounding of s and a: redo in FP64
            const double r64 = sqrt(fmax((double)r2.hi + (double)r2.lo, 0.0));
            v = (float)precession_average<double, false>(c, (double)s.hi + (double)s.lo, 0.0, r64 * c.phi,
                                                         nullptr, nullptr);
        }
        return v;
    }
    switch (c.shape) {
        case DS_SHAPE_LINEAR: {  // :52-73
            dd t = dd_sub(c.width_dd, dd_abs(s));
            float v = __fdiv_rn(t.hi + t.lo, c.width_f);
            return v > 0.f ? v : 0.f;
        }
        case DS_SHAPE_SINC:    // :76-101, s = 0 -> 0
        case DS_SHAPE_SIN2C: { // :104-123
            dd x = dd_mul(s, c.mw_dd);  // minima_number * s / width
            float v = 0.f;
            if (x.hi != 0.f) {
                float n = rintf(x.hi);
                float t = (x.hi - n) + x.lo;
                float sp = sinpif(t);
                v = fabsf(sp) / (3.14159265358979f * fabsf(x.hi + x.lo));
            }
            return c.shape == DS_SHAPE_SIN2C ? v * v : v;
        }
        default:
            return shape_base_f32(c, s.hi + s.lo);
    }
}

// shape factors, FP64 form (direct transcription)
template <bool INTEG>
__device__ inline double shape_fp64(const SimConst &c, double s, double r) {
    const double PI = 3.14159265358979323846;
    if (c.prec == DS_PRECESSION_LORENTZIAN) {
        double sigma = PI / c.width;
        double u = sigma * sigma * (r * r * c.phi * c.phi - s * s) + 1;
        double z = sqrt(u * u + 4 * sigma * sigma * s * s);
        return (sigma / PI) * sqrt(2 * (u + z) / (z * z));
    }
    if (INTEG) return precession_average<double, false>(c, s, 0.0, r * c.phi, nullptr, nullptr);
    return shape_base_f64(c, s);
}

struct TableP {
    const float4 *scr;
    const float *zh;
    const float4 *aux;    // per row, 32 bytes: the screen row (h, k, l, -z_mid), then |g|^2 as an FP32
                          // pair, |F|^2 (mixed), 0 -- one sector per candidate in the refine
    const double *F2d;
    const LineP *lines;   // line screen: per-line constants
    const int *line_meta; // [0] lines, [1] first trailing 000 row
    // brick screen: brick b holds up to 32 rows in slots [32 b, 32 b + 32):
    // their table rows bperm (-1: an empty slot), screen data bscr and bzh
    // (copies of scr and zh); brec[b] = (h, k, l of its block's centre,
    // -middle of its rows' z band), bhalf[b] = half width of that band plus
    // the block's radius; bmeta[0] = number of bricks
    const int32_t *bperm;
    const float4 *bscr;
    const float *bzh;
    const float4 *brec;
    const float *bhalf;
    const int32_t *bmeta;
};

// ------------------------------------------------------------- bricks ----
// The rows grouped into blocks of bh x bk x bl consecutive (h, k, l) of the
// table's index box.  A block's rows lie within rho (its corner radius,
// 1/Angstrom) of its centre g_c, and every row's z-interval [z_mid - z_half,
// z_mid + z_half] lies in the block's band [lo, hi]; with z = n . g and |n| =
// 1, a row can pass the per-row test only if |n . g_c - (lo + hi)/2| <
// (hi - lo)/2 + rho.  That test, widened by a rounding margin, is the brick
// test: rows of bricks that fail it are not tested.
struct BrickGeom {
    int bh, bk, bl;      // block edge in h, k, l
    int nbx, nby, nbz;   // blocks along h, k, l
    int hmax[3];
    float rho_margin;    // corner radius + rounding margin (1/Angstrom)
};
__host__ __device__ __forceinline__ int brick_block(const BrickGeom &G, int h, int k, int l) {
    // rows are within the box |h| <= hmax (the table's contract); clamped so
    // that a table breaking it cannot index outside the block arrays
    const int bx = min(max((h + G.hmax[0]) / G.bh, 0), G.nbx - 1);
    const int by = min(max((k + G.hmax[1]) / G.bk, 0), G.nby - 1);
    const int bz = min(max((l + G.hmax[2]) / G.bl, 0), G.nbz - 1);
    return (bx * G.nby + by) * G.nbz + bz;
}

// One candidate's table data, loaded ahead of its evaluation.
struct SpotIn {
    float4 e;    // h, k, l, -z_mid
    float2 g2;   // |g|^2 as an FP32 pair
    float F2;    // |F|^2 (mixed)
    double F2d;  // |F|^2 (FP64 form)
};
template <int FORM>
__device__ __forceinline__ SpotIn load_spot(const TableP &T, long long j) {
    SpotIn in;
    if (FORM == DS_FORM_FP64) {
        in.e = T.scr[j];
        in.F2d = T.F2d[j];
    } else {
        in.e = T.aux[2 * j];
        const float4 a = T.aux[2 * j + 1];
        in.g2 = make_float2(a.x, a.y);
        in.F2 = a.z;
    }
    return in;
}

// Evaluate one screened candidate: selection, intensity, beam-frame z.
template <int FORM, bool INTEG>
__device__ inline bool eval_in(const SimConst &c, const OrientP &op, const SpotIn &in, float &I, float &zout,
                               double &sout) {
    const float4 &e = in.e;
    if (FORM == DS_FORM_FP64) {
        double s, r, z;
        bool sel = select_fp64(c, op, (double)e.x, (double)e.y, (double)e.z, s, r, z);
        I = (float)(shape_fp64<INTEG>(c, s, r) * in.F2d);
        zout = (float)z;
        sout = s;
        return sel;
    } else {
        dd s, r2;
        float r, z;
        bool sel = select_mixed(c, op, e, in.g2, s, r, r2, z);
        I = shape_mixed<INTEG>(c, s, r, r2) * in.F2;
        zout = z;
        sout = (double)s.hi + (double)s.lo;
        return sel;
    }
}

template <int FORM, bool INTEG>
__device__ inline bool eval_spot(const SimConst &c, const OrientP &op, const TableP &T, long long j, float &I,
                                 float &zout, double &sout) {
    return eval_in<FORM, INTEG>(c, op, load_spot<FORM>(T, j), I, zout, sout);
}

template <int FORM>
__device__ __forceinline__ void spot_xy(const OrientP &op, const float4 &e, float &x, float &y) {
    if (FORM == DS_FORM_FP64) {
        x = (float)(op.M[0][0] * (double)e.x + op.M[0][1] * (double)e.y + op.M[0][2] * (double)e.z);
        y = (float)(op.M[1][0] * (double)e.x + op.M[1][1] * (double)e.y + op.M[1][2] * (double)e.z);
    } else {
        x = fmaf(op.m[0][0], e.x, fmaf(op.m[0][1], e.y, op.m[0][2] * e.z));
        y = fmaf(op.m[1][0], e.x, fmaf(op.m[1][1], e.y, op.m[1][2] * e.z));
    }
}

// 32x32 bit-matrix transpose across a warp: on return bit r of lane c is
// bit c of lane r on entry (recursive block swap, 5 butterfly stages).
__device__ __forceinline__ uint32_t transpose32(uint32_t x, int lane) {
    const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int w = 16 >> st;
        const uint32_t m = masks[st];
        const uint32_t y = __shfl_xor_sync(FULL_MASK, x, w);
        x = (lane & w) ? ((x & ~m) | ((y >> w) & m)) : ((x & m) | ((y << w) & ~m));
    }
    return x;
}

// Position of the n-th (0-based) set bit of w, n < popc(w): a popcount
// bisection over halves, quarters, ... (branch-free selects).
__device__ __forceinline__ int nth_set_bit(uint32_t w, int n) {
    int pos = 0, c;
    c = __popc(w & 0xFFFFu); if (n >= c) { n -= c; w >>= 16; pos += 16; }
    c = __popc(w & 0xFFu);   if (n >= c) { n -= c; w >>= 8;  pos += 8; }
    c = __popc(w & 0xFu);    if (n >= c) { n -= c; w >>= 4;  pos += 4; }
    c = __popc(w & 0x3u);    if (n >= c) { n -= c; w >>= 2;  pos += 2; }
    c = (int)(w & 1u);       if (n >= c) { pos += 1; }
    return pos;
}

__device__ __forceinline__ int owner_lane(int incl, int q) {
    int lo = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        int v = __shfl_sync(FULL_MASK, incl, lo + step - 1);
        if (v <= q) lo += step;
    }
    return lo;
}

// Iterate the set bits of bitmap words [w0, w1) of one orientation in row
// order, 32 at a time across the warp.  fn(j, rank, valid) is called by every
// lane (valid = lane holds a bit); rank = bit position in the ordered list.
template <typename Fn>
__device__ __forceinline__ void for_each_bit(const uint32_t *row, int w0, int w1, int lane, Fn fn) {
    int base_rank = 0;
    for (int g0 = w0; g0 < w1; g0 += 32) {
        int wi = g0 + lane;
        uint32_t word = wi < w1 ? row[wi] : 0u;
        int cnt = __popc(word);
        int incl = warp_inclusive_scan(cnt, lane);
        int total = __shfl_sync(FULL_MASK, incl, 31);
        for (int q0 = 0; q0 < total; q0 += 32) {
            int q = q0 + lane;
            bool valid = q < total;
            int own = owner_lane(incl, valid ? q : total - 1);
            uint32_t ow = __shfl_sync(FULL_MASK, word, own);
            int oin = __shfl_sync(FULL_MASK, incl, own);
            int bit = 0;
            if (valid) bit = nth_set_bit(ow, q - (oin - __popc(ow)));
            long long j = (long long)(g0 + own) * 32 + bit;
            fn(j, base_rank + q, valid, g0 + own, bit);
        }
        base_rank += total;
    }
}

// Set bits of bitmap words [w0, w1) of one orientation in row order, with K
// consecutive words per lane (groups of 32 K words) so sparse bitmaps still
// fill the lanes, and two candidates per lane per step (q and q + 32) so the
// table loads of both are in flight together.  fn(j0, rank0, valid0, j1,
// rank1, valid1) is called by every lane.
template <int K>
__device__ __forceinline__ void locate_bit(const uint32_t (&wd)[K], int incl, int cnt, int total, int q, int g0,
                                           long long &j, bool &valid) {
    valid = q < total;
    const int own = owner_lane(incl, valid ? q : total - 1);
    const int n = q - (__shfl_sync(FULL_MASK, incl, own) - __shfl_sync(FULL_MASK, cnt, own));
    uint32_t word = 0;
    int wsel = 0, before = 0, run = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const uint32_t ow = __shfl_sync(FULL_MASK, wd[k], own);
        const int pc = __popc(ow);
        if (n >= run && n < run + pc) { word = ow; wsel = k; before = run; }
        run += pc;
    }
    int bit = 0;
    if (valid) bit = nth_set_bit(word, n - before);
    j = (long long)(g0 + own * K + wsel) * 32 + bit;
}

template <int K, typename Fn>
__device__ __forceinline__ void for_each_bit_pair(const uint32_t *row, int w0, int w1, int lane, Fn fn) {
    int base_rank = 0;
    for (int g0 = w0; g0 < w1; g0 += 32 * K) {
        uint32_t wd[K];
        int cnt = 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int wi = g0 + lane * K + k;
            wd[k] = wi < w1 ? row[wi] : 0u;
            cnt += __popc(wd[k]);
        }
        const int incl = warp_inclusive_scan(cnt, lane);
        const int total = __shfl_sync(FULL_MASK, incl, 31);
        for (int q0 = 0; q0 < total; q0 += 64) {
            long long ja, jb;
            bool va, vb;
            locate_bit<K>(wd, incl, cnt, total, q0 + lane, g0, ja, va);
            locate_bit<K>(wd, incl, cnt, total, q0 + 32 + lane, g0, jb, vb);
            fn(ja, base_rank + q0 + lane, va, jb, base_rank + q0 + 32 + lane, vb);
        }
        base_rank += total;
    }
}

// Set bits of bitmap words [w0, w1) of one orientation in row order, as dense
// pairs: lanes append the rows of their own set bits to a per-warp queue in
// shared memory (their places known from one scan of the popcounts: no lane
// searches for its candidate), and full queues are evaluated one candidate
// per lane per round: load(j, valid) fetches a candidate's data, eval(j,
// rank, data) uses it.  A group denser than the queue is appended in
// several rounds.
template <int K, typename Load, typename Eval>
__device__ __forceinline__ void for_each_bit_queued(const uint32_t *row, int w0, int w1, int lane, int32_t *q,
                                                    Load load, Eval eval) {
    int qn = 0, rank_base = 0;
    // one candidate per lane per round; the next round's table data is
    // loaded before this round is evaluated, so the gather latency overlaps
    // the evaluation (one exposed latency per flush)
    auto flush = [&]() {
        __syncwarp();
        bool vc = lane < qn;
        long long jc = vc ? (long long)q[lane] : 0;
        auto cur = load(jc, vc);
        for (int r0 = 0; r0 < qn; r0 += 32) {
            const int rn = r0 + 32 + lane;
            const bool vn = rn < qn;
            const long long jn = vn ? (long long)q[rn] : 0;
            const auto nxt = load(jn, vn);
            if (vc) eval(jc, rank_base + r0 + lane, cur);
            cur = nxt;
            jc = jn;
            vc = vn;
        }
        rank_base += qn;
        qn = 0;
        __syncwarp();
    };
    for (int g0 = w0; g0 < w1; g0 += 32 * K) {
        uint32_t wd[K];
        int cnt = 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int wi = g0 + lane * K + k;
            wd[k] = wi < w1 ? row[wi] : 0u;
            cnt += __popc(wd[k]);
        }
        const int incl = warp_inclusive_scan(cnt, lane);
        const int total = __shfl_sync(FULL_MASK, incl, 31);
        int consumed = 0;
        while (consumed < total) {
            if (qn == SIM_QCAP) flush();
            const int take = min(SIM_QCAP - qn, total - consumed);
            int r = incl - cnt;  // group rank of this lane's first bit
#pragma unroll
            for (int k = 0; k < K; ++k) {
                uint32_t w = wd[k];
                const int wbase = (g0 + lane * K + k) * 32;
                while (w) {
                    const int b = __ffs(w) - 1;
                    w &= w - 1u;
                    if (r >= consumed && r < consumed + take) q[qn + r - consumed] = wbase + b;
                    ++r;
                }
            }
            qn += take;
            consumed += take;
        }
    }
    if (qn > 0) flush();
}

// Per-CTA staging in global scratch (L2-resident): the screened candidate
// rows of the tile in (orientation, row) order and their intensities, so the
// refine pass evaluates full warps of candidates once and the write pass
// only gathers.  Orientation parts that do not fit fall back to walking the
// bitmap and re-evaluating.
struct StageP {
    int32_t *idx;    // table row
    float *inten;    // I (-1: not a spot)
    long long cap;   // entries per pipeline slot
};
constexpr unsigned long long NO_STAGE = ~0ull;

// One phase of a batched launch: its candidate table, orientations and the
// per-phase geometry; tiles [tile0, tile0 + n_tiles) of the launch are its,
// its patterns are rows [orient0, orient0 + n_orient) of the output CSR.
struct PhaseP {
    TableP T;
    const double *quats;
    double recip[9];
    int hmax[3];
    int W, Ws;
    int O;  // orientations per tile of this phase (<= the kernel's O)
    long long n_hkl, n_orient, tile0, n_tiles, orient0;
};
constexpr int SIM_BATCH_MAX = 96;  // phases per launch (the descriptors travel as a kernel parameter)
struct PhaseBatch {
    int n;
    PhaseP ph[SIM_BATCH_MAX];
};

// f(integral_constant<int, v>) for v a power of two <= C (1 otherwise).
template <int C, class F>
__device__ __forceinline__ void dispatch_pow2(int v, F &f) {
    if constexpr (C <= 1) {
        f(std::integral_constant<int, 1>{});
    } else {
        if (v >= C) f(std::integral_constant<int, C>{});
        else dispatch_pow2<C / 2>(v, f);
    }
}

// The orientation kernel's body.  MULTI: many phases in one persistent
// launch, each tile of one phase; the phase's constants come from the batch
// descriptors (copied to shared memory per tile), the rest from c.
template <int O, int FORM, bool INTEG, bool MULTI>
__device__ __forceinline__ void simulate_body(const SimConst &c, const TableP &T1, const double *__restrict__ quats1,
                                              int64_t *__restrict__ offsets, int32_t *__restrict__ out_idx,
                                              float4 *__restrict__ out_xyzi, double *__restrict__ out_s,
                                              int64_t *__restrict__ out_total, LookbackScratch lb, StageP stg,
                                              int32_t *status, const PhaseP *batch, int n_batch) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ PhaseP s_ph[MULTI ? 2 : 1];
    const SimSmem Ls = sim_smem_layout(O, c.Ws);
    OrientP *sop_buf = reinterpret_cast<OrientP *>(smem + Ls.orient);                  // [2][O]
    unsigned long long *acc_buf = reinterpret_cast<unsigned long long *>(smem + Ls.acc);  // [2][ACC_STRIDE]
    uint32_t *bitmap = reinterpret_cast<uint32_t *>(smem + Ls.bitmap);                   // [O][Ws]
    int32_t *wqueue = reinterpret_cast<int32_t *>(smem + Ls.queue) + (threadIdx.x >> 5) * SIM_QCAP;
    __shared__ long long s_tile, s_prefix;
    __shared__ int s_defer;
    __shared__ int s_unit[4];  // work-unit counters of the dynamic phases

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int ACC_STRIDE = acc_stride(O);
    constexpr int ACC_TILE_TOTAL = O * ACC_WORDS;
    // phases 2-3 run over units (orientation, part): NP word ranges per
    // orientation (reflections per unit: the table over NP), taken by warps
    // from a shared counter for load balance; NP is a launch parameter
    const int NPL = c.parts_log2, NP = 1 << NPL;
    const bool all_zero_drop = c.zero_drop != 0;
    const unsigned lanemask_lt = (1u << lane) - 1u;
    auto part_range = [&](int Wp, int p, int &w0, int &w1) {
        w0 = (int)(((long long)Wp * p) >> NPL);
        w1 = (int)(((long long)Wp * (p + 1)) >> NPL);
    };
    // the phase constants of pipeline buffer b (one phase without MULTI)
    auto PW = [&](int b) -> int { return MULTI ? s_ph[b].W : c.W; };
    auto PWs = [&](int b) -> int { return MULTI ? s_ph[b].Ws : c.Ws; };
    auto PNH = [&](int b) -> long long { return MULTI ? s_ph[b].n_hkl : c.n_hkl; };
    auto PNO = [&](int b) -> long long { return MULTI ? s_ph[b].n_orient : c.n_orient; };
    auto PT0 = [&](int b) -> long long { return MULTI ? s_ph[b].tile0 : 0ll; };
    auto PO0 = [&](int b) -> long long { return MULTI ? s_ph[b].orient0 : 0ll; };
    auto PTab = [&](int b) -> const TableP & { return MULTI ? s_ph[b].T : T1; };
    auto POp = [&](int b) -> int { return MULTI ? s_ph[b].O : O; };
    auto next_unit = [&](int k) -> int {
        int u = 0;
        if (lane == 0) u = atomicAdd(&s_unit[k], 1);
        return __shfl_sync(FULL_MASK, u, 0);
    };

    // Two-stage software pipeline over tiles: a tile is screened and refined
    // (front), its count published, and its look-back and writes (back) run
    // after the NEXT tile's front, by when its predecessors have long
    // published: the look-back rarely waits.  Tiles whose candidates did not
    // all fit the staging need their bitmap in the back and are finished at
    // once.  Buffers (orientations, accumulators, staging) alternate.
    int cur = 0;
    long long pend_tile = -1;
    for (;;) {
        if (tid == 0) {
            const long long tk = (long long)atomicAdd(lb.ticket, 1ull);
            s_tile = tk;
            if (MULTI && tk < c.n_tiles) {
                // the phase holding this tile (tile0 ascends with the phase index)
                int lo = 0, hi = n_batch - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (batch[mid].tile0 <= tk) lo = mid;
                    else hi = mid - 1;
                }
                s_ph[cur] = batch[lo];
            }
        }
        if (tid < 4) s_unit[tid] = 0;
        OrientP *sop = sop_buf + cur * O;
        unsigned long long *acc = acc_buf + cur * ACC_STRIDE;
        int32_t *my_idx = stg.idx + (2 * (long long)blockIdx.x + cur) * stg.cap;
        float *my_I = stg.inten + (2 * (long long)blockIdx.x + cur) * stg.cap;
        for (int i = tid; i < ACC_STRIDE; i += SIM_THREADS)
            acc[i] = (i < ACC_TILE_TOTAL && i % ACC_WORDS == ACC_MINPOS) ? (unsigned long long)__float_as_uint(INFINITY)
                                                                          : 0ull;
        __syncthreads();
        const long long tile = s_tile;
        const bool have_new = tile < c.n_tiles;
        // the table pointers: kernel parameters for one phase; for many, a
        // register copy (a shared-memory reference would be reloaded at
        // every use)
        std::conditional_t<MULTI, const TableP, const TableP &> T = PTab(cur);
        const int W = PW(cur), Ws = PWs(cur);
        const long long n_hkl = PNH(cur);
        const int OP = POp(cur);  // this phase's tile (O without MULTI)
        const long long o_base = (tile - PT0(cur)) * OP;  // within the phase
        const int n_valid = have_new ? (int)min((long long)OP, PNO(cur) - o_base) : 0;
        const int n_units = n_valid * NP;
        if (have_new) {
            // ---------------- per-orientation rotation: beam frame = g @ R, R the active matrix of q
            // Orientation lane * 4 + warp on warps 0-3: the FP64 work (a warp
            // instruction holds its sub-partition's FP64 pipe for many
            // cycles whatever its active lanes) spread over the four SM
            // sub-partitions.
            const int orot = lane * 4 + warp;
            if (warp < 4 && orot < O) {
                OrientP &op = sop[orot];
                double R[3][3];
                if (orot < n_valid) {
                    const double *q = (MULTI ? s_ph[cur].quats : quats1) + 4 * (o_base + orot);
                    double w = q[0], x = q[1], y = q[2], z = q[3];
                    double nrm = sqrt(w * w + x * x + y * y + z * z);
                    if (!(nrm > 0) || !isfinite(nrm)) {
                        atomicOr(status, DS_ERR_NONFINITE);
                        nrm = 1; w = 1; x = y = z = 0;
                    }
                    const double inv = 1.0 / nrm;
                    w *= inv; x *= inv; y *= inv; z *= inv;
                    R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - w * z); R[0][2] = 2 * (x * z + w * y);
                    R[1][0] = 2 * (x * y + w * z); R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - w * x);
                    R[2][0] = 2 * (x * z - w * y); R[2][1] = 2 * (y * z + w * x); R[2][2] = 1 - 2 * (x * x + y * y);
                } else {
                    for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) R[a][b] = 0.0;
                }
                for (int cc = 0; cc < 3; ++cc)
                    for (int i = 0; i < 3; ++i) {
                        auto rc = [&](int k) -> double { return MULTI ? s_ph[cur].recip[k] : c.recip[k]; };
                        double v = rc(3 * i) * R[0][cc] + rc(3 * i + 1) * R[1][cc] + rc(3 * i + 2) * R[2][cc];
                        op.M[cc][i] = v;
                        op.m[cc][i] = (float)v;
                    }
                op.mz = make_float4(op.m[2][0], op.m[2][1], op.m[2][2], 0.f);
                // exact-product split of the z column: grid 2^q with 2^(q+24) >= 2 sum_i |M_zi| hmax_i
                double Z = 0.0;
                for (int i = 0; i < 3; ++i) Z += fabs(op.M[2][i]) * (double)(MULTI ? s_ph[cur].hmax[i] : c.hmax[i]);
                const int q = (Z > 0.0 ? ilogb(Z) : -100) + 2 - 24;
                for (int i = 0; i < 3; ++i) {
                    const double a = ldexp(rint(ldexp(op.M[2][i], -q)), q);
                    op.za[i] = (float)a;
                    op.zb[i] = (float)(op.M[2][i] - a);
                }
            }
            __syncthreads();

            // ---------------- phase 1: screen every row against all O orientations
            if (FORM == DS_FORM_MIXED && c.line_mode) {
                // per-(orientation, line) candidate intervals, OR-ed into a zeroed bitmap
                uint4 *bm4 = reinterpret_cast<uint4 *>(bitmap);
                for (int i = tid; i < (O * Ws + 3) / 4; i += SIM_THREADS) bm4[i] = make_uint4(0u, 0u, 0u, 0u);
                __syncthreads();
                const int n_lines = (int)min((long long)T.line_meta[0], n_hkl);  // bounded even if the line pass failed
                // trailing 000 rows: meta[1] holds the first one, or a large
                // sentinel when there are none
                const long long zero_start = min((long long)T.line_meta[1], n_hkl);
                const int n_zero = (int)(n_hkl - zero_start);  // 0, 1 or 2
                // the z rows in registers up to 16 orientations; above, one
                // broadcast shared load per use (3 O registers would spill)
                constexpr bool MREG = O <= 16;
                float mx[MREG ? O : 1], my[MREG ? O : 1], mz[MREG ? O : 1];
                if constexpr (MREG) {
#pragma unroll
                    for (int o = 0; o < O; ++o) { mx[o] = sop[o].m[2][0]; my[o] = sop[o].m[2][1]; mz[o] = sop[o].m[2][2]; }
                }
                for (int li = tid; li < n_lines; li += SIM_THREADS) {
                    const LineP L = T.lines[li];
#pragma unroll
                    for (int o = 0; o < O; ++o) {
                        if (o >= n_valid) continue;
                        if constexpr (MREG) {
                            line_candidates(c, L, mx[o], my[o], mz[o], bitmap + o * Ws);
                        } else {
                            const float4 m4 = sop[o].mz;
                            line_candidates(c, L, m4.x, m4.y, m4.z, bitmap + o * Ws);
                        }
                    }
                }
                // the trailing 000 rows (direct beam) are always candidates
                for (int i = tid; i < n_valid * n_zero; i += SIM_THREADS) {
                    const int o = i / n_zero;
                    const long long j = zero_start + i % n_zero;
                    atomicOr(&bitmap[o * Ws + (int)(j >> 5)], 1u << (int)(j & 31));
                }
            } else if (FORM == DS_FORM_MIXED && c.brick_mode) {
                // bricks: one test per (brick, orientation) with the lanes over
                // the tile's orientations; the brick's rows (lanes) are then
                // tested, exactly as the row screen tests them, for each
                // orientation the brick passes, and their bits or-ed into a
                // zeroed bitmap (the phase's OP rows) at their table positions.
                // A warp's bricks are b = warp + 8 i; the header and rows of the
                // next two are in flight while one is screened.
                uint4 *bm4 = reinterpret_cast<uint4 *>(bitmap);
                for (int i = tid; i < (OP * Ws + 3) / 4; i += SIM_THREADS) bm4[i] = make_uint4(0u, 0u, 0u, 0u);
                float b0 = 0.f, b1 = 0.f, b2 = 0.f;
                if (lane < n_valid) {
                    const float4 m4 = sop[lane].mz;
                    b0 = m4.x; b1 = m4.y; b2 = m4.z;
                }
                __syncthreads();
                const int nb = n_hkl > 0 ? T.bmeta[0] : 0;  // a phase without rows has no bricks
                struct BrickIn {
                    float4 h, e;
                    float hw, zh;
                    int j;
                };
                auto load_brick = [&](int b) {
                    BrickIn in;
                    in.h = make_float4(0.f, 0.f, 0.f, 0.f);
                    in.e = in.h;
                    in.hw = -1.f;
                    in.zh = -1.f;
                    in.j = -1;
                    if (b < nb) {
                        const long long slot = 32ll * b + lane;
                        in.h = T.brec[b];
                        in.hw = T.bhalf[b];
                        in.j = T.bperm[slot];
                        in.e = T.bscr[slot];
                        in.zh = T.bzh[slot];
                    }
                    return in;
                };
                BrickIn n0 = load_brick(warp), n1 = load_brick(warp + SIM_WARPS);
                for (int b = warp; b < nb; b += SIM_WARPS) {
                    const BrickIn cur = n0;
                    n0 = n1;
                    n1 = load_brick(b + 2 * SIM_WARPS);
                    const float zb = fmaf(b0, cur.h.x, fmaf(b1, cur.h.y, fmaf(b2, cur.h.z, cur.h.w)));
                    unsigned todo = __ballot_sync(FULL_MASK, lane < n_valid && fabsf(zb) < cur.hw);
                    while (todo) {
                        const int o = __ffs(todo) - 1;
                        todo &= todo - 1u;
                        const float4 m4 = sop[o].mz;
                        const float z = fmaf(m4.x, cur.e.x, fmaf(m4.y, cur.e.y, fmaf(m4.z, cur.e.z, cur.e.w)));
                        // the row screen's test: the sign of |z| - z_half
                        if (cur.j >= 0 && (__float_as_uint(fabsf(z) - cur.zh) >> 31) &&
                            DS_IN_BOUNDS(o * Ws + (cur.j >> 5), OP * Ws, status))
                            atomicOr(&bitmap[o * Ws + (cur.j >> 5)], 1u << (cur.j & 31));
                    }
                }
            } else if (FORM == DS_FORM_FP64) {
                for (int wc = warp; wc < W; wc += SIM_WARPS) {
                    const long long j = (long long)wc * 32 + lane;
                    float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (j < n_hkl) e = T.scr[j];
                    uint32_t myword = 0;
                    const double hd = e.x, kd = e.y, ld = e.z;
#pragma unroll 1
                    for (int o = 0; o < OP; ++o) {
                        double sx, rx, zx;
                        const bool hit = (j < n_hkl) && (o < n_valid) && select_fp64(c, sop[o], hd, kd, ld, sx, rx, zx);
                        const uint32_t b = __ballot_sync(FULL_MASK, hit);
                        if (lane == o) myword = b;
                    }
                    if (lane < OP && DS_IN_BOUNDS(lane * Ws + wc, O * Ws, status)) bitmap[lane * Ws + wc] = myword;
                }
            } else {
                constexpr bool MREG = O <= 16;  // as in the line screen
                float m0[MREG ? O : 1], m1[MREG ? O : 1], m2[MREG ? O : 1];
                if constexpr (MREG) {
#pragma unroll
                    for (int o = 0; o < O; ++o) { m0[o] = sop[o].m[2][0]; m1[o] = sop[o].m[2][1]; m2[o] = sop[o].m[2][2]; }
                }
                // Each step screens two chunks (wc, wc + 8) with independent
                // dependency chains; the rows of the next step are in flight.
                // Per orientation: the sign bit of |z - z_mid| - z_half, collected
                // into one word per lane (bit O-1-o); a 32x32 bit transpose then
                // hands lane O-1-o the word of orientation o.
                constexpr int CH = DS_SIM_SCREEN_CHUNKS;
                float4 en[CH];
                float zn[CH];
#pragma unroll
                for (int k = 0; k < CH; ++k) {
                    const long long jk = ((long long)warp + k * SIM_WARPS) * 32 + lane;
                    en[k] = make_float4(0.f, 0.f, 0.f, 0.f);
                    zn[k] = -1.f;
                    if (jk < n_hkl) { en[k] = T.scr[jk]; zn[k] = T.zh[jk]; }
                }
                // OPC: the tile's orientation count as a constant (a power of
                // two <= O; O without MULTI), so the unrolled per-orientation
                // chains carry no guard and interleave freely
                auto screen = [&](auto opc) {
                    constexpr int OPC = decltype(opc)::value;
                    for (int wc = warp; wc < W; wc += CH * SIM_WARPS) {
                        float4 e[CH];
                        float zh[CH];
#pragma unroll
                        for (int k = 0; k < CH; ++k) {
                            e[k] = en[k];
                            zh[k] = zn[k];
                            const long long jn = ((long long)wc + (CH + k) * SIM_WARPS) * 32 + lane;
                            en[k] = make_float4(0.f, 0.f, 0.f, 0.f);
                            zn[k] = -1.f;
                            if (jn < n_hkl) { en[k] = T.scr[jn]; zn[k] = T.zh[jn]; }
                        }
                        uint32_t bits[CH];
#pragma unroll
                        for (int k = 0; k < CH; ++k) bits[k] = 0;
#pragma unroll
                        for (int o = 0; o < OPC; ++o) {
                            float a0, a1, a2;
                            if constexpr (MREG) {
                                a0 = m0[o]; a1 = m1[o]; a2 = m2[o];
                            } else {
                                const float4 m4 = sop[o].mz;
                                a0 = m4.x; a1 = m4.y; a2 = m4.z;
                            }
#pragma unroll
                            for (int k = 0; k < CH; ++k) {
                                const float z = fmaf(a0, e[k].x, fmaf(a1, e[k].y, fmaf(a2, e[k].z, e[k].w)));
                                bits[k] = __funnelshift_l(__float_as_uint(fabsf(z) - zh[k]), bits[k], 1);
                            }
                        }
#pragma unroll
                        for (int k = 0; k < CH; ++k) bits[k] = transpose32(bits[k], lane);
#pragma unroll
                        for (int k = 0; k < CH; ++k) {
                            const int wck = wc + k * SIM_WARPS;
                            if (lane < OPC && wck < W && DS_IN_BOUNDS((OPC - 1 - lane) * Ws + wck, O * Ws, status))
                                bitmap[(OPC - 1 - lane) * Ws + wck] = bits[k];
                        }
                    }
                };
                if constexpr (!MULTI) screen(std::integral_constant<int, O>{});
                else dispatch_pow2<O>(OP, screen);
            }
            __syncthreads();

            // ---------------- candidate counts per unit and staging bases
            for (int u = warp; u < n_units; u += SIM_WARPS) {
                const int o = u >> NPL, p = u & (NP - 1);
                int w0, w1;
                part_range(W, p, w0, w1);
                const uint32_t *row = bitmap + o * Ws;
                int cnt = 0;
                for (int wi = w0 + lane; wi < w1; wi += 32) cnt += __popc(row[wi]);
#pragma unroll
                for (int d = 16; d >= 1; d >>= 1) cnt += __shfl_xor_sync(FULL_MASK, cnt, d);
                if (lane == 0) acc[o * ACC_WORDS + ACC_CCNT0 + p] = (unsigned long long)cnt;
            }
            __syncthreads();
            if (warp == 0) {
                // staging bases: the units in (orientation, part) order, the
                // longest prefix that fits the staging is staged
                constexpr int UPL_MAX = (O * 8 + 31) / 32;  // units per lane at NP = 8
                const int UPL = (O * NP + 31) / 32;
                long long cc[UPL_MAX], sum = 0;
#pragma unroll
                for (int i = 0; i < UPL_MAX; ++i) {
                    const int u = lane * UPL + i;
                    cc[i] = (i < UPL && u < n_units) ? (long long)acc[(u >> NPL) * ACC_WORDS + ACC_CCNT0 + (u & (NP - 1))]
                                                     : 0ll;
                    sum += cc[i];
                }
                long long run = warp_exclusive_scan_ll(sum, lane);
#pragma unroll
                for (int i = 0; i < UPL_MAX; ++i) {
                    const int u = lane * UPL + i;
                    if (i < UPL && u < n_units)
                        acc[(u >> NPL) * ACC_WORDS + ACC_CBASE0 + (u & (NP - 1))] =
                            run + cc[i] <= stg.cap ? (unsigned long long)run : NO_STAGE;
                    run += cc[i];
                }
            }
            __syncthreads();

            // ---------------- phase 2: refine, intensities, per-orientation max
            for (int u = next_unit(0); u < n_units; u = next_unit(0)) {
                const int o = u >> NPL, p = u & (NP - 1);
                int w0, w1;
                part_range(W, p, w0, w1);
                uint32_t *row = bitmap + o * Ws;
                const OrientP &op = sop[o];
                const unsigned long long base = acc[o * ACC_WORDS + ACC_CBASE0 + p];
                float lmax = 0.f, lminpos = INFINITY;
                int lcnt = 0;
                if (base != NO_STAGE) {
                    // evaluate each screened candidate once; stage (row, x, y, z, I)
                    // in candidate order, I = -1 for rejected candidates
                    for_each_bit_queued<4>(
                        row, w0, w1, lane, wqueue,
                        [&](long long j, bool v) {
                            SpotIn in;
                            if (v && DS_IN_BOUNDS(j, n_hkl, status)) in = load_spot<FORM>(T, j);
                            return in;
                        },
                        [&](long long j, int rk, const SpotIn &in) {
                            float I, z;
                            double sv;
                            bool sel = eval_in<FORM, INTEG>(c, op, in, I, z, sv);
                            if (sel && I == 0.f && all_zero_drop) sel = false;
                            if (DS_IN_BOUNDS(base + rk, stg.cap, status)) {
                                my_idx[base + rk] = (int32_t)j;
                                my_I[base + rk] = sel ? I : -1.f;
                            }
                            if (sel) {
                                ++lcnt;
                                lmax = fmaxf(lmax, I);
                                if (I > 0.f) lminpos = fminf(lminpos, I);
                            }
                        });
                } else {
                    for_each_bit(row, w0, w1, lane, [&](long long j, int, bool valid, int wi, int bit) {
                        if (!valid) return;
                        float I, z;
                        double sv;
                        bool sel = eval_spot<FORM, INTEG>(c, op, T, j, I, z, sv);
                        if (sel && I == 0.f && all_zero_drop) sel = false;
                        if (!sel) {
                            atomicAnd(&row[wi], ~(1u << bit));
                            return;
                        }
                        ++lcnt;
                        lmax = fmaxf(lmax, I);
                        if (I > 0.f) lminpos = fminf(lminpos, I);
                    });
                }
#pragma unroll
                for (int d = 16; d >= 1; d >>= 1) {
                    lmax = fmaxf(lmax, __shfl_xor_sync(FULL_MASK, lmax, d));
                    lminpos = fminf(lminpos, __shfl_xor_sync(FULL_MASK, lminpos, d));
                    lcnt += __shfl_xor_sync(FULL_MASK, lcnt, d);
                }
                if (!(lmax > 0.f)) lmax = 0.f;  // no -0.0 or NaN in the bit-ordered max
                if (lane == 0) {
                    // intensities are >= 0, so float bit patterns order like the values
                    atomicMax(&acc[o * ACC_WORDS + ACC_MAXI], (unsigned long long)__float_as_uint(lmax));
                    atomicMin(&acc[o * ACC_WORDS + ACC_MINPOS], (unsigned long long)__float_as_uint(lminpos));
                    acc[o * ACC_WORDS + ACC_PART0 + p] = (unsigned long long)lcnt;
                }
            }
            __syncthreads();

            // ---------------- mask pass (only where some I is positive but <= max * thr)
            bool need_mask = false;
            if (c.mask_on) {
                // FP32 first: t bounds max * thr from above unless it is near
                // the FP32 underflow; the exact FP64 test only where that
                // cannot decide (a warp-uniform branch: FP64 instructions are
                // scarce on this part and queue behind others)
                bool maybe = false;
                for (int o = lane; o < n_valid; o += 32) {
                    const float mx = __uint_as_float((unsigned)acc[o * ACC_WORDS + ACC_MAXI]);
                    const float mnp = __uint_as_float((unsigned)acc[o * ACC_WORDS + ACC_MINPOS]);
                    const float t = mx * c.thr_up;
                    maybe = maybe || !(mnp > t * 1.000002f) || t < 1e-30f;
                }
                if (__any_sync(FULL_MASK, maybe)) {
                    bool nm = false;
                    for (int o = lane; o < n_valid; o += 32) {
                        const float mx = __uint_as_float((unsigned)acc[o * ACC_WORDS + ACC_MAXI]);
                        const float mnp = __uint_as_float((unsigned)acc[o * ACC_WORDS + ACC_MINPOS]);
                        nm = nm || (double)mnp <= (double)mx * c.thr;
                    }
                    need_mask = __any_sync(FULL_MASK, nm);
                }
            }
            if (need_mask) {
                for (int u = next_unit(1); u < n_units; u = next_unit(1)) {
                    const int o = u >> NPL, p = u & (NP - 1);
                    const float mx = __uint_as_float((unsigned)acc[o * ACC_WORDS + ACC_MAXI]);
                    const float mnp = __uint_as_float((unsigned)acc[o * ACC_WORDS + ACC_MINPOS]);
                    if (!((double)mnp <= (double)mx * c.thr)) continue;
                    int w0, w1;
                    part_range(W, p, w0, w1);
                    uint32_t *row = bitmap + o * Ws;
                    const OrientP &op = sop[o];
                    const unsigned long long base = acc[o * ACC_WORDS + ACC_CBASE0 + p];
                    const int cc = (int)acc[o * ACC_WORDS + ACC_CCNT0 + p];
                    int dropped = 0;
                    if (base != NO_STAGE) {
                        for (int r = lane; r < cc; r += 32) {
                            const float I = my_I[base + r];
                            if (!(I < 0.f) && !((double)I > (double)mx * c.thr)) {
                                my_I[base + r] = -1.f;
                                ++dropped;
                            }
                        }
                    } else {
                        for_each_bit(row, w0, w1, lane, [&](long long j, int, bool valid, int wi, int bit) {
                            if (!valid) return;
                            float I, z;
                            double sv;
                            eval_spot<FORM, INTEG>(c, op, T, j, I, z, sv);
                            if (!((double)I > (double)mx * c.thr)) {
                                atomicAnd(&row[wi], ~(1u << bit));
                                ++dropped;
                            }
                        });
                    }
#pragma unroll
                    for (int d = 16; d >= 1; d >>= 1) dropped += __shfl_xor_sync(FULL_MASK, dropped, d);
                    if (lane == 0) acc[o * ACC_WORDS + ACC_PART0 + p] -= (unsigned long long)dropped;
                }
                __syncthreads();
            }

            // ---------------- tile count, published for the look-back of later tiles
            if (warp == 0) {
                // per orientation (one lane each; O <= 32): kept count and
                // offset within the tile; the tile total, published
                long long co = 0;
                bool staged = true;
                if (lane < n_valid) {
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        co += (long long)acc[lane * ACC_WORDS + ACC_PART0 + p];
                        staged = staged && acc[lane * ACC_WORDS + ACC_CBASE0 + p] != NO_STAGE;
                    }
                }
                const long long excl = warp_exclusive_scan_ll(co, lane);
                if (lane < n_valid) {
                    acc[lane * ACC_WORDS + ACC_OFF] = (unsigned long long)excl;
                    acc[lane * ACC_WORDS + ACC_CNT] = (unsigned long long)co;
                }
                const long long run = __shfl_sync(FULL_MASK, excl + co, 31);
                const bool defer = __all_sync(FULL_MASK, staged);
                if (lane == 0) {
                    acc[ACC_TILE_TOTAL] = (unsigned long long)run;
                    lookback_publish(lb, tile, run);
                    s_defer = defer ? 1 : 0;
                }
            }
            __syncthreads();
        }  // have_new

        // ---------------- back: look-back and ordered writes of a finished tile
        auto back = [&](long long btile, int bbuf, int counter) -> bool {
            const OrientP *bsop = sop_buf + bbuf * O;
            const unsigned long long *bacc = acc_buf + bbuf * ACC_STRIDE;
            const int32_t *b_idx = stg.idx + (2 * (long long)blockIdx.x + bbuf) * stg.cap;
            const float *b_I = stg.inten + (2 * (long long)blockIdx.x + bbuf) * stg.cap;
            std::conditional_t<MULTI, const TableP, const TableP &> T = PTab(bbuf);
            const int W = PW(bbuf), Ws = PWs(bbuf);
            const int BOP = POp(bbuf);
            const long long bo_base = (btile - PT0(bbuf)) * BOP;
            const long long bo_out = PO0(bbuf) + bo_base;  // first output row of the tile
            const int bn_valid = (int)min((long long)BOP, PNO(bbuf) - bo_base);
            if (tid == 0) {
                const long long run = (long long)bacc[ACC_TILE_TOTAL];
                const long long prefix = lookback_resolve(lb, btile, run, status);
                s_prefix = prefix;
                if (prefix >= 0 && btile == c.n_tiles - 1) {
                    offsets[c.n_orient] = prefix + run;
                    *out_total = prefix + run;
                }
            }
            __syncthreads();
            const long long prefix = s_prefix;
            if (prefix < 0) return false;  // bounded wait gave up: DS_ERR_TIMEOUT is set
            for (int o = tid; o < bn_valid; o += SIM_THREADS)
                offsets[bo_out + o] = prefix + (long long)bacc[o * ACC_WORDS + ACC_OFF];
            for (int u = next_unit(counter); u < bn_valid * NP; u = next_unit(counter)) {
                const int o = u >> NPL, p = u & (NP - 1);
                int w0, w1;
                part_range(W, p, w0, w1);
                const uint32_t *row = bitmap + o * Ws;
                const OrientP &op = bsop[o];
                long long pos0 = prefix + (long long)bacc[o * ACC_WORDS + ACC_OFF];
                for (int pp = 0; pp < p; ++pp) pos0 += (long long)bacc[o * ACC_WORDS + ACC_PART0 + pp];
                const unsigned long long base = bacc[o * ACC_WORDS + ACC_CBASE0 + p];
                const int cc = (int)bacc[o * ACC_WORDS + ACC_CCNT0 + p];
                bool overflow = false;
                if (base != NO_STAGE) {
                    // compaction of the staged (row, I) pairs, four batches in flight;
                    // beam-frame x, y, z recomputed from the row's hkl
                    long long out_r = 0;
                    for (int r0 = 0; r0 < cc; r0 += 128) {
                        float II[4];
                        int32_t jj[4];
#pragma unroll
                        for (int b = 0; b < 4; ++b) {
                            const int r = r0 + 32 * b + lane;
                            II[b] = -1.f;
                            jj[b] = 0;
                            if (r < cc && DS_IN_BOUNDS(base + r, stg.cap, status)) {
                                II[b] = b_I[base + r];
                                jj[b] = b_idx[base + r];
                            }
                        }
                        float4 ee[4];
#pragma unroll
                        for (int b = 0; b < 4; ++b) {
                            ee[b] = make_float4(0.f, 0.f, 0.f, 0.f);
                            if (!(II[b] < 0.f) && DS_IN_BOUNDS(jj[b], PNH(bbuf), status)) ee[b] = T.scr[jj[b]];
                        }
#pragma unroll
                        for (int b = 0; b < 4; ++b) {
                            const bool keep = !(II[b] < 0.f);
                            const unsigned bal = __ballot_sync(FULL_MASK, keep);
                            if (keep) {
                                const float4 e = ee[b];
                                float x, y, z;
                                spot_xy<FORM>(op, e, x, y);
                                if (FORM == DS_FORM_FP64)
                                    z = (float)(op.M[2][0] * (double)e.x + op.M[2][1] * (double)e.y + op.M[2][2] * (double)e.z);
                                else
                                    z = fmaf(op.za[0], e.x, fmaf(op.za[1], e.y, op.za[2] * e.z)) +
                                        fmaf(op.zb[0], e.x, fmaf(op.zb[1], e.y, op.zb[2] * e.z));
                                const long long pos = pos0 + out_r + __popc(bal & lanemask_lt);
                                if (pos < c.capacity) {
                                    if (c.idx16)
                                        reinterpret_cast<uint16_t *>(out_idx)[pos] = (uint16_t)jj[b];
                                    else
                                        out_idx[pos] = jj[b];
                                    out_xyzi[pos] = make_float4(x, y, z, II[b]);
                                    if (out_s) {
                                        float I2, z2;
                                        double sv;
                                        eval_spot<FORM, INTEG>(c, op, T, jj[b], I2, z2, sv);
                                        out_s[pos] = sv;
                                    }
                                } else {
                                    overflow = true;
                                }
                            }
                            out_r += __popc(bal);
                        }
                    }
                } else {
                    for_each_bit(row, w0, w1, lane, [&](long long j, int rank, bool valid, int, int) {
                        if (!valid) return;
                        float I, z;
                        double sv;
                        eval_spot<FORM, INTEG>(c, op, T, j, I, z, sv);
                        const float4 e = T.scr[j];
                        float x, y;
                        spot_xy<FORM>(op, e, x, y);
                        const long long pos = pos0 + rank;
                        if (pos < c.capacity) {
                            if (c.idx16)
                                reinterpret_cast<uint16_t *>(out_idx)[pos] = (uint16_t)j;
                            else
                                out_idx[pos] = (int32_t)j;
                            out_xyzi[pos] = make_float4(x, y, z, I);
                            if (out_s) out_s[pos] = sv;
                        } else {
                            overflow = true;
                        }
                    });
                }
                if (__any_sync(FULL_MASK, overflow) && lane == 0) atomicOr(status, DS_ERR_CAPACITY);
            }
            __syncthreads();  // staging / bitmap reused afterwards
            return true;
        };

        if (pend_tile >= 0) {
            if (!back(pend_tile, cur ^ 1, 2)) break;
            pend_tile = -1;
        }
        if (!have_new) break;
        if (s_defer) {
            pend_tile = tile;
            cur ^= 1;
        } else if (!back(tile, cur, 3)) {
            break;
        }
    }
}

template <int O, int FORM, bool INTEG>
__global__ void __launch_bounds__(SIM_THREADS, 2)
simulate_kernel(SimConst c, TableP T, const double *__restrict__ quats, int64_t *__restrict__ offsets,
                int32_t *__restrict__ out_idx, float4 *__restrict__ out_xyzi, double *__restrict__ out_s,
                int64_t *__restrict__ out_total, LookbackScratch lb, StageP stg, int32_t *status) {
    simulate_body<O, FORM, INTEG, false>(c, T, quats, offsets, out_idx, out_xyzi, out_s, out_total, lb, stg, status,
                                         nullptr, 0);
}

// Many phases in one persistent launch: the tile ticket runs over the phases'
// tiles in order and the look-back orders the output across phases.
template <int O, int FORM, bool INTEG>
__global__ void __launch_bounds__(SIM_THREADS, 2)
simulate_batch_kernel(SimConst c, const __grid_constant__ PhaseBatch B, int64_t *__restrict__ offsets,
                      int32_t *__restrict__ out_idx, float4 *__restrict__ out_xyzi, double *__restrict__ out_s,
                      int64_t *__restrict__ out_total, LookbackScratch lb, StageP stg, int32_t *status) {
    simulate_body<O, FORM, INTEG, true>(c, B.ph[0].T, nullptr, offsets, out_idx, out_xyzi, out_s, out_total, lb, stg,
                                        status, B.ph, B.n);
}

// ----------------------------------------------------------- host helpers ----
// Dynamic shared memory one CTA may take with two CTAs resident per SM (the
// occupancy the kernels are built for), less a margin for static shared data.
inline long long sim_two_cta_smem() {
    int dev = 0, per_sm = 0, reserved = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess)
        return 100 * 1024;
    return (long long)per_sm / 2 - reserved - 512;
}

// Argument checks shared by the single-phase and batched entries.
inline ds_status validate_params(const ds_sim_params *p, const char *who) {
    const std::string w(who);
    DS_REQUIRE(p->k0 > 0 && isfinite(p->k0), w + ": k0 must be finite and > 0");
    DS_REQUIRE(p->max_excitation_error > 0 && isfinite(p->max_excitation_error),
               w + ": max_excitation_error must be > 0");
    DS_REQUIRE(p->shape_width != 0 && isfinite(p->shape_width), w + ": shape width must be finite, non-zero");
    DS_REQUIRE(p->shape_model >= DS_SHAPE_LINEAR && p->shape_model <= DS_SHAPE_BINARY, w + ": bad shape model");
    DS_REQUIRE(p->precession_mode >= DS_PRECESSION_NONE && p->precession_mode <= DS_PRECESSION_INTEGRAL,
               w + ": bad precession mode");
    DS_REQUIRE(p->form == DS_FORM_MIXED || p->form == DS_FORM_FP64, w + ": bad form");
    DS_REQUIRE(p->orient_tile == 0 || p->orient_tile == 1 || p->orient_tile == 2 || p->orient_tile == 4 ||
                   p->orient_tile == 8 || p->orient_tile == 16 || p->orient_tile == 32,
               w + ": orient_tile must be 0, 1, 2, 4, 8, 16 or 32");
    DS_REQUIRE(p->stage_cap >= 0, w + ": stage_cap < 0");
    DS_REQUIRE(p->refine_parts == 0 || p->refine_parts == 1 || p->refine_parts == 2 || p->refine_parts == 4 ||
                   p->refine_parts == 8,
               w + ": refine_parts must be 0, 1, 2, 4 or 8");
    DS_REQUIRE(p->precession_mode == DS_PRECESSION_NONE || p->precession_angle > 0,
               w + ": precession mode needs a positive angle");

    return DS_OK;
}

// log2 of the refine / write units per orientation: the caller's choice, or
// two per orientation (eight for single-orientation tiles, so the units still
// fill the CTA's warps).
inline int refine_parts_log2(const ds_sim_params *p, int O) {
    const int parts = p->refine_parts > 0 ? p->refine_parts : (O >= 2 ? 2 : 8);
    return parts >= 8 ? 3 : parts >= 4 ? 2 : parts >= 2 ? 1 : 0;
}

// The kernel constants of one phase; the per-launch fields (O, W, Ws,
// n_orient, n_tiles, capacity, line_mode, parts_log2) are set by the caller.
inline void fill_const(const ds_sim_params *p, const ds_phase_table *t, SimConst &c) {
    c.idx16 = 0;
    c.k0 = p->k0;
    c.eps = p->max_excitation_error;
    c.width = p->shape_width;
    c.phi = p->precession_angle;
    c.thr = p->minimum_intensity;
    c.mask_on = c.thr > 0.0;
    c.zero_drop = c.thr >= 0.0;
    c.thr_up = std::nextafter((float)(c.thr * (1.0 + 1e-6)), INFINITY);
    c.minima = p->minima_number;
    c.Pz = p->k0 * cos(p->precession_angle);
    c.Pt = p->k0 * sin(p->precession_angle);
    for (int i = 0; i < 9; ++i) c.recip[i] = t->recip[i];
    split_double(c.eps, c.eps_dd.hi, c.eps_dd.lo);
    split_double(1.0 / (2.0 * c.k0), c.c2k0_dd.hi, c.c2k0_dd.lo);
    split_double(c.width, c.width_dd.hi, c.width_dd.lo);
    split_double(c.minima / c.width, c.mw_dd.hi, c.mw_dd.lo);
    split_double(c.phi, c.phi_dd.hi, c.phi_dd.lo);
    const double PI = 3.14159265358979323846;
    c.k0f = (float)c.k0;
    c.inv_k0sq = (float)(1.0 / (c.k0 * c.k0));
    c.eps_f = (float)c.eps;
    c.width_f = (float)c.width;
    c.sigma_f = (float)(PI / c.width);
    c.mfac_f = (float)(PI * c.minima / fabs(c.width));
    c.phi_f = (float)c.phi;
    c.Pz_f = (float)c.Pz;
    c.Pt_f = (float)c.Pt;
    c.k0sq_f = (float)(c.k0 * c.k0);
    c.mw_f = (float)(c.minima / c.width);
    c.int_step = precession_breakpoint_step(p->shape_model, c.width, c.minima);
    c.int_step_f = (float)c.int_step;
    c.int_tau = precession_fp64_threshold(p->shape_model);
    // FP32 screen guard: bound on |z32 - z| from rounding m to FP32 and the FMA
    // chain, 8 ulp of sum_i |row_i of recip| * max|hkl_i| (|R| = 1), plus the
    // rounding of z_mid and z_half.
    double zmax = 0;
    for (int i = 0; i < 3; ++i)
        zmax += sqrt(t->recip[3 * i] * t->recip[3 * i] + t->recip[3 * i + 1] * t->recip[3 * i + 1] +
                     t->recip[3 * i + 2] * t->recip[3 * i + 2]) * (double)t->hmax[i];
    c.guard = (float)(8.0 * 5.96e-8 * zmax + 4.0 * 5.96e-8 * (c.eps + zmax * zmax / (2 * c.k0)) + 1e-7);
    c.shape = p->shape_model;
    c.prec = p->precession_mode;
    c.form = p->form;
    for (int i = 0; i < 3; ++i) c.hmax[i] = t->hmax[i] > 0 ? t->hmax[i] : 1;
    c.n_hkl = t->n_hkl;
    {
        const double e = c.eps, k0 = c.k0;
        c.alpha1 = 1.0 / (2.0 * (k0 - e));
        c.alpha0 = (e * e - 2.0 * e * k0) * c.alpha1;
        c.beta1 = 1.0 / (2.0 * (k0 + e));
        c.beta0 = (e * e + 2.0 * e * k0) * c.beta1;
        c.csq = t->recip[6] * t->recip[6] + t->recip[7] * t->recip[7] + t->recip[8] * t->recip[8];
        c.a2f = (float)(-c.alpha1 * c.csq);
        c.b2f = (float)(-c.beta1 * c.csq);
        c.inv_a2f = 1.f / c.a2f;
        c.inv_b2f = 1.f / c.b2f;
    }
    c.O = 0;
    c.W = (int)((t->n_hkl + 31) / 32);
    c.Ws = c.W | 1;
    c.n_orient = 0;
    c.line_mode = 0;
    c.brick_mode = 0;
    c.parts_log2 = 1;
    c.n_tiles = 0;
    c.capacity = 0;
}

// sim_prep_kernel launcher (simulate.cu): the screen arrays of one table.
ds_status launch_sim_prep(const SimConst &c, const int32_t *hkl, const double *g2, const float *F2, float4 *scr, float *zh, float4 *aux,
                          long long n_hkl, cudaStream_t s);

// Brick screen (simulate.cu).  brick_geometry picks the block shape for a
// table (recip rows a*, b*, c*; hmax) and a tile of O orientations, whose
// selection band reaches `reach` (1/Angstrom) off the Ewald sphere;
// brick_scratch_bytes is the scratch the bricks of n rows take;
// launch_brick_build fills the brick arrays of T from the table rows and the
// prep's screen arrays (after launch_sim_prep, on the same stream).
BrickGeom brick_geometry(const double recip[9], const int32_t hmax[3], int O, double reach);
double selection_reach(const ds_sim_params *p, const ds_phase_table *t);
size_t brick_scratch_bytes(const BrickGeom &G, long long n_hkl);
ds_status launch_brick_build(const BrickGeom &G, const int32_t *hkl, long long n_hkl, const float4 *scr,
                             const float *zh, void *scratch, TableP &T, cudaStream_t s);

// ------------------------------------------------------------- host side ----

// Kernel entry of (O, FORM) with the precession rotation average compiled in
// (simulate_integral.cu); the other instantiations live in simulate.cu.
const void *simulate_kernel_integral(int O, int form);
// Batched entries (simulate_batch.cu, simulate_batch_integral.cu); O in {1, 2,
// 4, 8, 16} (mixed) or {1, 2, 4, 8} (FP64).
const void *simulate_batch_kernel_plain(int O, int form);
const void *simulate_batch_kernel_integral(int O, int form);

}  // namespace ds
