// Adjoint of the spot intensities I = shf(s, r) |F_hkl|^2 (no counterpart in
// the reference, which is not differentiable): given dL/dI for every spot of a
// forward ds_simulate call, the gradients of L with respect to the structure
// (fractional coordinates, occupancies, Debye-Waller B), the reciprocal basis
// (hence the lattice parameters) and the orientations.
//
//   ds_simulate_backward           one warp per orientation walks its spots:
//       FP64 geometry g = B*^T h, u = R^T g, r, s (the forward's formulas);
//       shape factor and its partials in s and r (closed forms; the precession
//       average by the forward's quadrature with f' on the same nodes);
//       dL/d|F|^2 per row (atomic FP64), dL/dR per orientation (warp sum),
//       dL/dB* from the geometry (warp sums, 9 atomics per warp).
//   ds_structure_factors_backward  recomputes F_hkl (FP64; structure factors
//       are never stored per orientation), then per (atom, chunk of rows) sums
//       dL/d|F|^2 * d|F|^2/d(x, occ, B), and dL/dB* through |g|^2 (scattering
//       factors and Debye-Waller) per row.
// The forward is FP32 with FP64 phase reduction; the adjoint is FP64 except
// the precession-average quadrature (FP32, FP64 below 1e-2 as in the forward).
#include <math.h>

#include <algorithm>

#include "common.cuh"
#include "shape.cuh"

namespace ds {

constexpr int BW_THREADS = 256;

struct BwdConst {
    int shape, prec;
    double width, minima, phi, int_step, k0;
    float width_f, mw_f, mfac_f, sigma_f, phi_f, int_step_f, int_tau;
    double recip[9];
    long long n_orient, n_hkl;
};

__device__ inline void quat_matrix(const double *q, double R[3][3]) {
    double w = q[0], x = q[1], y = q[2], z = q[3];
    double nrm = sqrt(w * w + x * x + y * y + z * z);
    if (!(nrm > 0) || !isfinite(nrm)) {
        nrm = 1; w = 1; x = y = z = 0;
    }
    w /= nrm; x /= nrm; y /= nrm; z /= nrm;
    R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - w * z); R[0][2] = 2 * (x * z + w * y);
    R[1][0] = 2 * (x * y + w * z); R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - w * x);
    R[2][0] = 2 * (x * z - w * y); R[2][1] = 2 * (y * z + w * x); R[2][2] = 1 - 2 * (x * x + y * y);
}

// dL/dq of R(q / |q|) from G = dL/dR (row-major): dL/dq^ = sum G . dR/dq^,
// then the projection through the normalisation, (g - (q^.g) q^) / |q|.
__device__ inline void quat_adjoint(const double *q, const double (&G)[9], double *out) {
    double w = q[0], x = q[1], y = q[2], z = q[3];
    double nrm = sqrt(w * w + x * x + y * y + z * z);
    if (!(nrm > 0) || !isfinite(nrm)) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return;
    }
    w /= nrm; x /= nrm; y /= nrm; z /= nrm;
    const double gw = 2 * (-z * G[1] + y * G[2] + z * G[3] - x * G[5] - y * G[6] + x * G[7]);
    const double gx = 2 * (y * G[1] + z * G[2] + y * G[3] - 2 * x * G[4] - w * G[5] + z * G[6] + w * G[7] - 2 * x * G[8]);
    const double gy = 2 * (-2 * y * G[0] + x * G[1] + w * G[2] + x * G[3] + z * G[5] - w * G[6] + z * G[7] - 2 * y * G[8]);
    const double gz = 2 * (-2 * z * G[0] - w * G[1] + x * G[2] + w * G[3] - 2 * z * G[4] + y * G[5] + x * G[6] + y * G[7]);
    const double dot = w * gw + x * gx + y * gy + z * gz;
    out[0] = (gw - dot * w) / nrm;
    out[1] = (gx - dot * x) / nrm;
    out[2] = (gy - dot * y) / nrm;
    out[3] = (gz - dot * z) / nrm;
}

// q = q0 (x) exp(v): Hamilton product with the unit quaternion of the rotation
// vector v (angle |v|), and its adjoint in v.
__device__ inline void axis_angle_quat(const double *v, double e[4], double &k, double &th) {
    th = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double sh, ch;
    sincos(0.5 * th, &sh, &ch);
    k = th < 1e-6 ? 0.5 - th * th / 48.0 : sh / th;  // sin(th/2) / th
    e[0] = ch;
    e[1] = k * v[0];
    e[2] = k * v[1];
    e[3] = k * v[2];
}

__global__ void axis_angle_compose_kernel(const double *__restrict__ q0, const double *__restrict__ v, long long n,
                                          double *__restrict__ q) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double e[4], k, th;
    axis_angle_quat(v + 3 * i, e, k, th);
    const double *p = q0 + 4 * i;
    q[4 * i + 0] = p[0] * e[0] - p[1] * e[1] - p[2] * e[2] - p[3] * e[3];
    q[4 * i + 1] = p[0] * e[1] + p[1] * e[0] + p[2] * e[3] - p[3] * e[2];
    q[4 * i + 2] = p[0] * e[2] - p[1] * e[3] + p[2] * e[0] + p[3] * e[1];
    q[4 * i + 3] = p[0] * e[3] + p[1] * e[2] - p[2] * e[1] + p[3] * e[0];
}

__global__ void axis_angle_compose_backward_kernel(const double *__restrict__ q0, const double *__restrict__ v,
                                                   long long n, const double *__restrict__ gq,
                                                   double *__restrict__ gv) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double e[4], k, th;
    const double *vi = v + 3 * i;
    axis_angle_quat(vi, e, k, th);
    const double *p = q0 + 4 * i, *g = gq + 4 * i;
    // q = L(p) e: dL/de = L(p)^T dL/dq
    const double ge0 = p[0] * g[0] + p[1] * g[1] + p[2] * g[2] + p[3] * g[3];
    const double ge1 = -p[1] * g[0] + p[0] * g[1] + p[3] * g[2] - p[2] * g[3];
    const double ge2 = -p[2] * g[0] - p[3] * g[1] + p[0] * g[2] + p[1] * g[3];
    const double ge3 = -p[3] * g[0] + p[2] * g[1] - p[1] * g[2] + p[0] * g[3];
    // e = (cos(th/2), k(th) v): de0/dv = -sin(th/2)/(2 th) v, de_j/dv_i = k d_ij + (k'/th) v_i v_j
    double a0, kp;  // -sin(th/2)/(2 th), k'(th)/th
    if (th < 1e-3) {
        a0 = -0.25 + th * th / 96.0;
        kp = -1.0 / 24.0 + th * th / 960.0;
    } else {
        double sh, ch;
        sincos(0.5 * th, &sh, &ch);
        a0 = -sh / (2.0 * th);
        kp = (0.5 * th * ch - sh) / (th * th * th);
    }
    const double gdv = ge1 * vi[0] + ge2 * vi[1] + ge3 * vi[2];
    const double common = ge0 * a0 + kp * gdv;
    gv[3 * i + 0] = vi[0] * common + k * ge1;
    gv[3 * i + 1] = vi[1] * common + k * ge2;
    gv[3 * i + 2] = vi[2] * common + k * ge3;
}

// shf and its partial derivatives in s and r at one spot.
template <int PREC>
__device__ inline double shape_and_grad(const BwdConst &c, double s, double r, double &ds, double &dr) {
    if (PREC == DS_PRECESSION_LORENTZIAN) return lorentzian_precession_grad(c, s, r, ds, dr);
    if (PREC == DS_PRECESSION_INTEGRAL) {
        float sh, sl, d0, da;
        split_double(s, sh, sl);
        float v = precession_average_inline<float, true>(c, sh, sl, (float)(r * c.phi), &d0, &da);
        if (v < c.int_tau) {
            double e0, ea;
            double vd = precession_average_inline<double, true>(c, s, 0.0, r * c.phi, &e0, &ea);
            ds = e0;
            dr = ea * c.phi;
            return vd;
        }
        ds = (double)d0;
        dr = (double)da * c.phi;
        return (double)v;
    }
    ds = shape_deriv<double>(c, s);
    dr = 0.0;
    return shape_base_f64(c, s);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) v += __shfl_xor_sync(FULL_MASK, v, d);
    return v;
}

// Per-orientation constants of the adjoint: R (the active rotation of the
// normalised quaternion) and M = R^T B*^T, with u = M h the beam-frame g.  The
// z row stays FP64 (s is a cancellation: k0 - sqrt(k0^2 - r^2) - z), the
// rest is FP32.
struct OrientB {
    double Mz[3];
    float M[3][3], R[3][3];
};
__device__ __forceinline__ void orient_setup(const BwdConst &c, const double *q, OrientB &O) {
    double R[3][3];
    quat_matrix(q, R);
#pragma unroll
    for (int cc = 0; cc < 3; ++cc)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double m = R[0][cc] * c.recip[3 * i] + R[1][cc] * c.recip[3 * i + 1] + R[2][cc] * c.recip[3 * i + 2];
            O.M[cc][i] = (float)m;
            if (cc == 2) O.Mz[i] = m;
        }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) O.R[k][cc] = (float)R[k][cc];
}

// Beam-frame geometry of one spot: z in FP64, r^2 = |g|^2 - z^2 in FP64 (no
// cancellation), k0 - sqrt(k0^2 - r^2) = r^2 / (k0 + sqrt(k0^2 - r^2)) in FP32
// (relative 1e-7 of a term <= r^2 / 2k0), s = that - z in FP64: |ds| ~ 1e-9.
struct SpotGeom {
    float h[3], u[3];
    float r, rt;
    double s;
};
__device__ __forceinline__ void spot_geometry(const BwdConst &c, const OrientB &O, const int32_t *hkl,
                                              const double *g2, int row, SpotGeom &G) {
    const int hi = hkl[3 * row], ki = hkl[3 * row + 1], li = hkl[3 * row + 2];
    G.h[0] = (float)hi;
    G.h[1] = (float)ki;
    G.h[2] = (float)li;
    const double z = O.Mz[0] * (double)hi + O.Mz[1] * (double)ki + O.Mz[2] * (double)li;
#pragma unroll
    for (int cc = 0; cc < 2; ++cc) G.u[cc] = fmaf(O.M[cc][0], G.h[0], fmaf(O.M[cc][1], G.h[1], O.M[cc][2] * G.h[2]));
    G.u[2] = (float)z;
    const float r2 = (float)fmax(g2[row] - z * z, 0.0);
    G.r = sqrtf(r2);
    G.rt = sqrtf((float)(c.k0 * c.k0) - r2);
    G.s = (double)(r2 / ((float)c.k0 + G.rt)) - z;
}

// Precession rotation average: the shape factor and its partials of every
// spot, in their own pass (the quadrature needs registers the accumulating
// pass holds for its sums), one thread per spot for balance (the quadrature's
// cost varies with the spot's radius): part[j] = (shf, d shf / d s, d shf / d r).
// The orientation constants come from orient_prep_kernel.
__global__ void orient_prep_kernel(const BwdConst c, const double *__restrict__ quats, OrientB *__restrict__ ob) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= c.n_orient) return;
    OrientB O;
    orient_setup(c, quats + 4 * o, O);
    ob[o] = O;
}

__global__ void __launch_bounds__(BW_THREADS)
shape_partials_kernel(const BwdConst c, const OrientB *__restrict__ ob, const int64_t *__restrict__ offsets,
                      const int32_t *__restrict__ hkl_index, const int32_t *__restrict__ hkl,
                      const double *__restrict__ g2, long long n_spots, double *__restrict__ part, int32_t *status) {
    const long long total = min((long long)offsets[c.n_orient], n_spots);
    if (blockIdx.x == 0 && threadIdx.x == 0 && offsets[c.n_orient] > n_spots) atomicOr(status, DS_ERR_CAPACITY);
    for (long long j = (long long)blockIdx.x * BW_THREADS + threadIdx.x; j < total;
         j += (long long)gridDim.x * BW_THREADS) {
        // orientation of spot j: last o with offsets[o] <= j
        long long lo = 0, hi = c.n_orient - 1;
        while (lo < hi) {
            const long long mid = (lo + hi + 1) >> 1;
            if (offsets[mid] <= j) lo = mid;
            else hi = mid - 1;
        }
        const OrientB O = ob[lo];
        SpotGeom G;
        spot_geometry(c, O, hkl, g2, hkl_index[j], G);
        double ds, dr;
        const double shf = shape_and_grad<DS_PRECESSION_INTEGRAL>(c, G.s, (double)G.r, ds, dr);
        part[3 * j] = shf;
        part[3 * j + 1] = ds;
        part[3 * j + 2] = dr;
    }
}

// Accumulation: per spot FP32 products, per orientation FP64 sums.
template <int PREC, bool PRE>
__global__ void __launch_bounds__(BW_THREADS)
spot_backward_kernel(const BwdConst c, const double *__restrict__ quats, const int64_t *__restrict__ offsets,
                     const int32_t *__restrict__ hkl_index, const double *__restrict__ grad_I,
                     const int32_t *__restrict__ hkl, const double *__restrict__ g2, const float *__restrict__ F2,
                     const double *__restrict__ F2d, const double *__restrict__ part, long long n_spots,
                     double *__restrict__ grad_F2, double *__restrict__ grad_q, double *__restrict__ grad_recip) {
    const int lane = threadIdx.x & 31;
    const long long warp0 = ((long long)blockIdx.x * BW_THREADS + threadIdx.x) >> 5;
    const long long n_warps = ((long long)gridDim.x * BW_THREADS) >> 5;
    double gB[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) gB[i] = 0.0;
    for (long long o = warp0; o < c.n_orient; o += n_warps) {
        OrientB O;
        orient_setup(c, quats + 4 * o, O);
        float gR[9], gBo[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) gR[i] = gBo[i] = 0.f;
        const long long a = offsets[o], b = min((long long)offsets[o + 1], n_spots);
        for (long long j = a + lane; j < b; j += 32) {
            const int row = hkl_index[j];
            SpotGeom G;
            spot_geometry(c, O, hkl, g2, row, G);
            double dsh_ds, dsh_dr, shf;
            if (PRE) {
                shf = part[3 * j];
                dsh_ds = part[3 * j + 1];
                dsh_dr = part[3 * j + 2];
            } else {
                shf = shape_and_grad<PREC>(c, G.s, (double)G.r, dsh_ds, dsh_dr);
            }
            const double f2 = F2d ? F2d[row] : (double)F2[row];
            const double gI = grad_I[j];
            atomicAdd(grad_F2 + row, gI * shf);
            const float as = (float)(gI * f2 * dsh_ds), ar = (float)(gI * f2 * dsh_dr);
            float du[3];
            du[2] = -as;  // s = k0 - sqrt(k0^2 - r^2) - u_z
            if (G.r > 0.f) {
                const float dLdr = fmaf(as, G.r / G.rt, ar);
                const float ir = 1.f / G.r;
                du[0] = dLdr * G.u[0] * ir;
                du[1] = dLdr * G.u[1] * ir;
            } else {
                du[0] = du[1] = 0.f;
            }
            // u = R^T g: dL/dR[k][c] = du_c g_k; dL/dg_k = sum_c R[k][c] du_c;
            // g = B*^T h: dL/dB*[i][k] = h_i dL/dg_k
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float gk = G.h[0] * (float)c.recip[k] + G.h[1] * (float)c.recip[3 + k] +
                                 G.h[2] * (float)c.recip[6 + k];
                float dg = 0.f;
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) {
                    gR[3 * k + cc] = fmaf(du[cc], gk, gR[3 * k + cc]);
                    dg = fmaf(O.R[k][cc], du[cc], dg);
                }
#pragma unroll
                for (int i = 0; i < 3; ++i) gBo[3 * i + k] = fmaf(G.h[i], dg, gBo[3 * i + k]);
            }
        }
        double G[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            G[i] = warp_sum((double)gR[i]);
            gB[i] += (double)gBo[i];
        }
        if (lane == 0) quat_adjoint(quats + 4 * o, G, grad_q + 4 * o);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const double v = warp_sum(gB[i]);
        if (lane == 0 && v != 0.0) atomicAdd(grad_recip + i, v);
    }
}

// ------------------------------------------------ structure-factor adjoint ----
struct SfbConst {
    long long n;
    int n_atoms, n_species, kind, _pad;
    double recip[9];
};

// f_s(g^2) and d f_s / d g^2 (diffsims/utils/sim_utils.py:249-253)
__device__ inline double scatter_and_grad(const double *cf, int kind, double g2, double &df) {
    df = 0.0;
    if (kind == DS_SCATTER_NONE) return 1.0;
    double f = 0.0;
    for (int i = 0; i < 5; ++i) {
        const double a = cf[2 * i], b = cf[2 * i + 1];
        const double gb = g2 * b;
        if (kind == DS_SCATTER_LOBATO) {
            const double d = 1.0 + gb;
            f += a * (2.0 + gb) / (d * d);
            df += a * b * (-3.0 - gb) / (d * d * d);
        } else {
            const double e = exp(-0.25 * gb);
            f += a * e;
            df += -0.25 * b * a * e;
        }
    }
    return f;
}

// sin and cos of 2 pi h.x: the phase reduced modulo 1 in FP64 (as in the
// forward), then FP32 sincospi.  The adjoint's products are FP32, its sums
// FP64: a term's rounding is relative to that term, so every gradient
// component keeps ~1e-7 of the largest contribution.
__device__ __forceinline__ void phase_sc(double hx, float &sn, float &cs) {
    const double t = hx - rint(hx);
    sincospif((float)(2.0 * t), &sn, &cs);
}

// Per row: f_s(g^2) and d f_s / d g^2 of every species (FP64, stored for the
// per-atom pass); F = (Re, Im); dL/d|g|^2 through the scattering factors and
// Debye-Waller; its share of dL/dB* (|g|^2 = |B*^T h|^2).
__global__ void __launch_bounds__(BW_THREADS)
sf_rows_backward_kernel(const SfbConst c, const ds_atoms A, const int32_t *__restrict__ hkl,
                        const double *__restrict__ g2v, const double *__restrict__ grad_F2,
                        double2 *__restrict__ F, double2 *__restrict__ fs_tab, double *__restrict__ grad_recip) {
    __shared__ double s_red[BW_THREADS / 32][9];
    const long long j = (long long)blockIdx.x * BW_THREADS + threadIdx.x;
    double gB[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) gB[i] = 0.0;
    if (j < c.n) {
        const double h = hkl[3 * j], k = hkl[3 * j + 1], l = hkl[3 * j + 2];
        const double g2 = g2v[j];
        for (int sp = 0; sp < c.n_species; ++sp) {
            double dfs;
            const double fs = scatter_and_grad(A.coeffs + 10 * sp, c.kind, g2, dfs);
            fs_tab[(long long)sp * c.n + j] = make_double2(fs, dfs);
        }
        double re = 0, im = 0, dre = 0, dim = 0;
        for (int a = 0; a < c.n_atoms; ++a) {
            const ds_atom at = A.atoms[a];
            const double2 f = fs_tab[(long long)at.species * c.n + j];
            const float dw = expf((float)(-0.25 * at.B * g2));
            const float amp = (float)(at.occupancy * f.x) * dw;
            const float damp = (float)(at.occupancy * (f.y - 0.25 * at.B * f.x)) * dw;  // d amp / d g^2
            float sn, cs;
            phase_sc(h * at.x + k * at.y + l * at.z, sn, cs);
            re += (double)(amp * cs);
            im += (double)(amp * sn);
            dre += (double)(damp * cs);
            dim += (double)(damp * sn);
        }
        F[j] = make_double2(re, im);
        const double dLdg2 = grad_F2[j] * 2.0 * (re * dre + im * dim);
        const double hv[3] = {h, k, l};
        double g[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) g[q] = h * c.recip[q] + k * c.recip[3 + q] + l * c.recip[6 + q];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int q = 0; q < 3; ++q) gB[3 * i + q] = dLdg2 * 2.0 * g[q] * hv[i];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const double v = warp_sum(gB[i]);
        if (lane == 0) s_red[w][i] = v;
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        double v = 0.0;
        for (int q = 0; q < BW_THREADS / 32; ++q) v += s_red[q][threadIdx.x];
        if (v != 0.0) atomicAdd(grad_recip + threadIdx.x, v);
    }
}

constexpr int SFB_CHUNK = 64;  // rows per thread in the per-atom pass

// Per (atom, chunk of rows): sum over rows of dL/d|F|^2 * d|F|^2 / d(x, y, z, occ, B).
__global__ void __launch_bounds__(BW_THREADS)
sf_atoms_backward_kernel(const SfbConst c, const ds_atoms A, const int32_t *__restrict__ hkl,
                         const double *__restrict__ g2v, const double *__restrict__ grad_F2,
                         const double2 *__restrict__ F, const double2 *__restrict__ fs_tab,
                         double *__restrict__ grad_atoms) {
    const long long t = (long long)blockIdx.x * BW_THREADS + threadIdx.x;
    const long long n_chunks = (c.n + SFB_CHUNK - 1) / SFB_CHUNK;
    if (t >= n_chunks * c.n_atoms) return;
    const int a = (int)(t % c.n_atoms);
    const long long j0 = (t / c.n_atoms) * SFB_CHUNK;
    const long long j1 = min(j0 + SFB_CHUNK, c.n);
    const ds_atom at = A.atoms[a];
    const double2 *fsa = fs_tab + (long long)at.species * c.n;
    const double TWO_PI = 6.283185307179586476925;
    const float mq = (float)(-0.25 * at.B);
    double gx = 0, gy = 0, gz = 0, gocc = 0, gb = 0;
    for (long long j = j0; j < j1; ++j) {
        const double G = grad_F2[j];
        if (G == 0.0) continue;
        const double h = hkl[3 * j], k = hkl[3 * j + 1], l = hkl[3 * j + 2];
        const double g2 = g2v[j];
        const float fs = (float)fsa[j].x;
        const float dw = expf(mq * (float)g2);
        const float amp = (float)at.occupancy * fs * dw;
        float sn, cs;
        phase_sc(h * at.x + k * at.y + l * at.z, sn, cs);
        const double2 Fj = F[j];
        // |F|^2 = Re^2 + Im^2, Re = sum amp cos, Im = sum amp sin
        const double px = 2.0 * ((double)(amp * cs) * Fj.y - (double)(amp * sn) * Fj.x) * TWO_PI;  // d|F|^2/d(h.x)
        gx += G * px * h;
        gy += G * px * k;
        gz += G * px * l;
        const double pc = 2.0 * (Fj.x * (double)cs + Fj.y * (double)sn);  // d|F|^2 / d amp
        gocc += G * pc * (double)(fs * dw);
        gb += G * pc * (double)amp * (-0.25 * g2);
    }
    double *o = grad_atoms + 5 * a;
    atomicAdd(o + 0, gx);
    atomicAdd(o + 1, gy);
    atomicAdd(o + 2, gz);
    atomicAdd(o + 3, gocc);
    atomicAdd(o + 4, gb);
}

}  // namespace ds

using namespace ds;

extern "C" size_t ds_simulate_backward_scratch_bytes(const ds_sim_params *p, int64_t n_spots, int64_t n_orient) {
    if (!p || n_spots < 0 || n_orient <= 0 || p->precession_mode != DS_PRECESSION_INTEGRAL) return 0;
    return (((size_t)n_spots * 3 * sizeof(double) + 255) / 256) * 256 + (size_t)n_orient * sizeof(OrientB);
}

extern "C" ds_status ds_simulate_backward(const ds_sim_params *p, const ds_phase_table *t, const double *quats,
                                          int64_t n_orient, const int64_t *offsets, const int32_t *hkl_index,
                                          int64_t n_spots, const double *grad_intensity, double *grad_F2,
                                          double *grad_quats, double *grad_recip, void *scratch, size_t scratch_bytes,
                                          int32_t *status, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_simulate_backward");
    DS_REQUIRE(p && t, "ds_simulate_backward: null pointer");
    DS_REQUIRE(n_orient >= 0, "ds_simulate_backward: n_orient < 0");
    DS_REQUIRE(p->k0 > 0 && isfinite(p->k0), "ds_simulate_backward: k0 must be finite and > 0");
    DS_REQUIRE(p->shape_width != 0 && isfinite(p->shape_width), "ds_simulate_backward: bad shape width");
    DS_REQUIRE(p->shape_model >= DS_SHAPE_LINEAR && p->shape_model <= DS_SHAPE_BINARY,
               "ds_simulate_backward: bad shape model");
    DS_REQUIRE(p->precession_mode >= DS_PRECESSION_NONE && p->precession_mode <= DS_PRECESSION_INTEGRAL,
               "ds_simulate_backward: bad precession mode");
    DS_REQUIRE(n_spots >= 0, "ds_simulate_backward: n_spots < 0");
    if (n_orient == 0) return DS_OK;
    DS_REQUIRE(quats && offsets && grad_F2 && grad_quats && grad_recip && status, "ds_simulate_backward: null array");
    DS_REQUIRE(n_spots == 0 || (hkl_index && grad_intensity), "ds_simulate_backward: null spot arrays");
    DS_REQUIRE(scratch_bytes >= ds_simulate_backward_scratch_bytes(p, n_spots, n_orient) &&
                   (ds_simulate_backward_scratch_bytes(p, n_spots, n_orient) == 0 || scratch),
               "ds_simulate_backward: scratch too small");
    DS_REQUIRE(t->n_hkl == 0 || (t->hkl && t->g2 && (t->F2 || t->F2d)), "ds_simulate_backward: table arrays missing");
    BwdConst c;
    c.shape = p->shape_model;
    c.prec = p->precession_mode;
    c.width = p->shape_width;
    c.minima = p->minima_number;
    c.phi = p->precession_angle;
    c.k0 = p->k0;
    c.int_step = precession_breakpoint_step(p->shape_model, c.width, c.minima);
    const double PI = 3.14159265358979323846;
    c.width_f = (float)c.width;
    c.mw_f = (float)(c.minima / c.width);
    c.mfac_f = (float)(PI * c.minima / fabs(c.width));
    c.sigma_f = (float)(PI / c.width);
    c.phi_f = (float)c.phi;
    c.int_step_f = (float)c.int_step;
    c.int_tau = precession_fp64_threshold_quadrature(p->shape_model);
    for (int i = 0; i < 9; ++i) c.recip[i] = t->recip[i];
    c.n_orient = n_orient;
    c.n_hkl = t->n_hkl;
    int dev = 0, n_sm = 0;
    DS_CUDA_TRY(cudaGetDevice(&dev));
    DS_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    const long long want = (n_orient * 32 + BW_THREADS - 1) / BW_THREADS;
    const int grid = (int)std::min<long long>(want, (long long)n_sm * 8);
    const double *F2d = (p->form == DS_FORM_FP64 && t->F2d) ? t->F2d : nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    const long long ns = n_spots;
    if (c.prec == DS_PRECESSION_INTEGRAL) {
        double *part = reinterpret_cast<double *>(scratch);
        OrientB *ob = reinterpret_cast<OrientB *>(reinterpret_cast<unsigned char *>(scratch) +
                                                  (((size_t)ns * 3 * sizeof(double) + 255) / 256) * 256);
        orient_prep_kernel<<<(unsigned)((n_orient + 127) / 128), 128, 0, s>>>(c, quats, ob);
        ds_status st = check_launch("orient_prep_kernel");
        if (st) return st;
        const long long pblocks = std::min<long long>((ns + BW_THREADS - 1) / BW_THREADS, (long long)n_sm * 16);
        if (ns > 0) {
            shape_partials_kernel<<<(unsigned)std::max(1ll, pblocks), BW_THREADS, 0, s>>>(c, ob, offsets, hkl_index,
                                                                                         t->hkl, t->g2, ns, part,
                                                                                         status);
            st = check_launch("shape_partials_kernel");
            if (st) return st;
        }
        spot_backward_kernel<DS_PRECESSION_INTEGRAL, true><<<grid, BW_THREADS, 0, s>>>(
            c, quats, offsets, hkl_index, grad_intensity, t->hkl, t->g2, t->F2, F2d, part, ns, grad_F2, grad_quats, grad_recip);
    } else if (c.prec == DS_PRECESSION_LORENTZIAN) {
        spot_backward_kernel<DS_PRECESSION_LORENTZIAN, false><<<grid, BW_THREADS, 0, s>>>(
            c, quats, offsets, hkl_index, grad_intensity, t->hkl, t->g2, t->F2, F2d, nullptr, ns, grad_F2, grad_quats, grad_recip);
    } else {
        spot_backward_kernel<DS_PRECESSION_NONE, false><<<grid, BW_THREADS, 0, s>>>(
            c, quats, offsets, hkl_index, grad_intensity, t->hkl, t->g2, t->F2, F2d, nullptr, ns, grad_F2, grad_quats, grad_recip);
    }
    return check_launch("spot_backward_kernel");
}

extern "C" size_t ds_structure_factors_backward_scratch_bytes(int64_t n, int32_t n_species) {
    if (n <= 0 || n_species < 0) return 0;
    return (size_t)n * sizeof(double2) * (size_t)(1 + n_species);
}

extern "C" ds_status ds_structure_factors_backward(const ds_atoms *atoms, const int32_t *hkl, const double *g2,
                                                   int64_t n, const double recip[9], const double *grad_F2,
                                                   double *grad_atoms, double *grad_recip, void *scratch,
                                                   size_t scratch_bytes, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_structure_factors_backward");
    DS_REQUIRE(atoms && recip, "ds_structure_factors_backward: null pointer");
    DS_REQUIRE(n >= 0, "ds_structure_factors_backward: n < 0");
    DS_REQUIRE(atoms->n_atoms >= 0 && atoms->n_species >= 0 && atoms->n_species <= 32,
               "ds_structure_factors_backward: bad atom counts");
    DS_REQUIRE(atoms->kind == DS_SCATTER_LOBATO || atoms->kind == DS_SCATTER_XTABLES || atoms->kind == DS_SCATTER_NONE,
               "ds_structure_factors_backward: bad scattering kind");
    if (n == 0 || atoms->n_atoms == 0) return DS_OK;
    DS_REQUIRE(hkl && g2 && grad_F2 && grad_atoms && grad_recip && atoms->atoms,
               "ds_structure_factors_backward: null array");
    DS_REQUIRE(atoms->kind == DS_SCATTER_NONE || atoms->coeffs, "ds_structure_factors_backward: null coefficients");
    DS_REQUIRE(scratch && scratch_bytes >= ds_structure_factors_backward_scratch_bytes(n, atoms->n_species),
               "ds_structure_factors_backward: scratch too small");
    SfbConst c;
    c.n = n;
    c.n_atoms = atoms->n_atoms;
    c.n_species = atoms->n_species;
    c.kind = atoms->kind;
    c._pad = 0;
    for (int i = 0; i < 9; ++i) c.recip[i] = recip[i];
    cudaStream_t s = (cudaStream_t)stream;
    double2 *F = reinterpret_cast<double2 *>(scratch);
    double2 *fs_tab = F + n;
    sf_rows_backward_kernel<<<(unsigned)((n + BW_THREADS - 1) / BW_THREADS), BW_THREADS, 0, s>>>(
        c, *atoms, hkl, g2, grad_F2, F, fs_tab, grad_recip);
    ds_status st = check_launch("sf_rows_backward_kernel");
    if (st) return st;
    const long long n_chunks = (n + SFB_CHUNK - 1) / SFB_CHUNK;
    const long long threads = n_chunks * atoms->n_atoms;
    sf_atoms_backward_kernel<<<(unsigned)((threads + BW_THREADS - 1) / BW_THREADS), BW_THREADS, 0, s>>>(
        c, *atoms, hkl, g2, grad_F2, F, fs_tab, grad_atoms);
    return check_launch("sf_atoms_backward_kernel");
}

extern "C" ds_status ds_axis_angle_compose(const double *q0, const double *rotvec, int64_t n, double *quats_out,
                                           void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_axis_angle_compose");
    DS_REQUIRE(n >= 0, "ds_axis_angle_compose: n < 0");
    if (n == 0) return DS_OK;
    DS_REQUIRE(q0 && rotvec && quats_out, "ds_axis_angle_compose: null array");
    axis_angle_compose_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(q0, rotvec, n, quats_out);
    return check_launch("axis_angle_compose_kernel");
}

extern "C" ds_status ds_axis_angle_compose_backward(const double *q0, const double *rotvec, int64_t n,
                                                    const double *grad_quats, double *grad_rotvec, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_axis_angle_compose_backward");
    DS_REQUIRE(n >= 0, "ds_axis_angle_compose_backward: n < 0");
    if (n == 0) return DS_OK;
    DS_REQUIRE(q0 && rotvec && grad_quats && grad_rotvec, "ds_axis_angle_compose_backward: null array");
    axis_angle_compose_backward_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        q0, rotvec, n, grad_quats, grad_rotvec);
    return check_launch("axis_angle_compose_backward_kernel");
}
