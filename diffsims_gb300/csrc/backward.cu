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
constexpr float BW_TAU_INT = 1e-2f;

struct BwdConst {
    int shape, prec;
    double width, minima, phi, int_step, k0;
    float width_f, mw_f, mfac_f, sigma_f, phi_f, int_step_f;
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

// shf and its partial derivatives in s and r at one spot.
template <int PREC>
__device__ inline double shape_and_grad(const BwdConst &c, double s, double r, double &ds, double &dr) {
    if (PREC == DS_PRECESSION_LORENTZIAN) return lorentzian_precession_grad(c, s, r, ds, dr);
    if (PREC == DS_PRECESSION_INTEGRAL) {
        float sh, sl, d0, da;
        split_double(s, sh, sl);
        float v = precession_average_inline<float, true>(c, sh, sl, (float)(r * c.phi), &d0, &da);
        if (v < BW_TAU_INT) {
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

template <int PREC>
__global__ void __launch_bounds__(BW_THREADS)
spot_backward_kernel(const BwdConst c, const double *__restrict__ quats, const int64_t *__restrict__ offsets,
                     const int32_t *__restrict__ hkl_index, const double *__restrict__ grad_I,
                     const int32_t *__restrict__ hkl, const float *__restrict__ F2, const double *__restrict__ F2d,
                     double *__restrict__ grad_F2, double *__restrict__ grad_R, double *__restrict__ grad_recip) {
    const int lane = threadIdx.x & 31;
    const long long warp0 = ((long long)blockIdx.x * BW_THREADS + threadIdx.x) >> 5;
    const long long n_warps = ((long long)gridDim.x * BW_THREADS) >> 5;
    double gB[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) gB[i] = 0.0;
    const double k0sq = c.k0 * c.k0;
    for (long long o = warp0; o < c.n_orient; o += n_warps) {
        double R[3][3];
        quat_matrix(quats + 4 * o, R);
        double gR[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) gR[i] = 0.0;
        const long long a = offsets[o], b = offsets[o + 1];
        for (long long j = a + lane; j < b; j += 32) {
            const int row = hkl_index[j];
            const double hi[3] = {(double)hkl[3 * row], (double)hkl[3 * row + 1], (double)hkl[3 * row + 2]};
            double g[3], u[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) g[k] = hi[0] * c.recip[k] + hi[1] * c.recip[3 + k] + hi[2] * c.recip[6 + k];
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) u[cc] = R[0][cc] * g[0] + R[1][cc] * g[1] + R[2][cc] * g[2];
            const double r = sqrt(u[0] * u[0] + u[1] * u[1]);
            const double rt = sqrt(k0sq - r * r);
            const double s = (-rt + c.k0) - u[2];
            double dsh_ds, dsh_dr;
            const double shf = shape_and_grad<PREC>(c, s, r, dsh_ds, dsh_dr);
            const double f2 = F2d ? F2d[row] : (double)F2[row];
            const double gI = grad_I[j];
            atomicAdd(grad_F2 + row, gI * shf);
            const double as = gI * f2 * dsh_ds, ar = gI * f2 * dsh_dr;
            double du[3];
            du[2] = -as;  // s = k0 - sqrt(k0^2 - r^2) - u_z
            if (r > 0.0) {
                const double dLdr = ar + as * (r / rt);
                du[0] = dLdr * u[0] / r;
                du[1] = dLdr * u[1] / r;
            } else {
                du[0] = du[1] = 0.0;
            }
            // u = R^T g: dL/dR[k][c] = du_c g_k; dL/dg_k = sum_c R[k][c] du_c;
            // g = B*^T h: dL/dB*[i][k] = h_i dL/dg_k
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double dg = 0.0;
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) {
                    gR[3 * k + cc] += du[cc] * g[k];
                    dg += R[k][cc] * du[cc];
                }
#pragma unroll
                for (int i = 0; i < 3; ++i) gB[3 * i + k] += hi[i] * dg;
            }
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const double v = warp_sum(gR[i]);
            if (lane == 0) grad_R[9 * o + i] = v;
        }
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

// reduced phase of h.x (FP64): sin and cos of 2 pi h.x
__device__ __forceinline__ void phase_sc(double hx, double &sn, double &cs) {
    const double t = hx - rint(hx);
    sincospi(2.0 * t, &sn, &cs);
}

// Per row: F = (Re, Im) recomputed in FP64 and stored; dL/d|g|^2 through the
// scattering factors and Debye-Waller; its share of dL/dB* (|g|^2 = |B*^T h|^2).
__global__ void __launch_bounds__(BW_THREADS)
sf_rows_backward_kernel(const SfbConst c, const ds_atoms A, const int32_t *__restrict__ hkl,
                        const double *__restrict__ g2v, const double *__restrict__ grad_F2,
                        double2 *__restrict__ F, double *__restrict__ grad_recip) {
    __shared__ double s_red[BW_THREADS / 32][9];
    const long long j = (long long)blockIdx.x * BW_THREADS + threadIdx.x;
    double gB[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) gB[i] = 0.0;
    if (j < c.n) {
        const double h = hkl[3 * j], k = hkl[3 * j + 1], l = hkl[3 * j + 2];
        const double g2 = g2v[j];
        double re = 0, im = 0, dre = 0, dim = 0;
        for (int a = 0; a < c.n_atoms; ++a) {
            const ds_atom at = A.atoms[a];
            double dfs;
            const double fs = scatter_and_grad(A.coeffs + 10 * at.species, c.kind, g2, dfs);
            const double dw = exp(-0.25 * at.B * g2);
            const double amp = at.occupancy * fs * dw;
            const double damp = at.occupancy * dw * (dfs - 0.25 * at.B * fs);  // d amp / d g^2
            double sn, cs;
            phase_sc(h * at.x + k * at.y + l * at.z, sn, cs);
            re += amp * cs;
            im += amp * sn;
            dre += damp * cs;
            dim += damp * sn;
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
                         const double2 *__restrict__ F, double *__restrict__ grad_atoms) {
    const long long t = (long long)blockIdx.x * BW_THREADS + threadIdx.x;
    const long long n_chunks = (c.n + SFB_CHUNK - 1) / SFB_CHUNK;
    if (t >= n_chunks * c.n_atoms) return;
    const int a = (int)(t % c.n_atoms);
    const long long j0 = (t / c.n_atoms) * SFB_CHUNK;
    const long long j1 = min(j0 + SFB_CHUNK, c.n);
    const ds_atom at = A.atoms[a];
    const double *cf = A.coeffs + 10 * at.species;
    const double TWO_PI = 6.283185307179586476925;
    double gx = 0, gy = 0, gz = 0, gocc = 0, gb = 0;
    for (long long j = j0; j < j1; ++j) {
        const double G = grad_F2[j];
        if (G == 0.0) continue;
        const double h = hkl[3 * j], k = hkl[3 * j + 1], l = hkl[3 * j + 2];
        const double g2 = g2v[j];
        double dfs;
        const double fs = scatter_and_grad(cf, c.kind, g2, dfs);
        const double dw = exp(-0.25 * at.B * g2);
        const double amp = at.occupancy * fs * dw;
        double sn, cs;
        phase_sc(h * at.x + k * at.y + l * at.z, sn, cs);
        const double2 Fj = F[j];
        // |F|^2 = Re^2 + Im^2, Re = sum amp cos, Im = sum amp sin
        const double px = 2.0 * (Fj.y * amp * cs - Fj.x * amp * sn) * TWO_PI;  // d|F|^2 / d(h.x)
        gx += G * px * h;
        gy += G * px * k;
        gz += G * px * l;
        const double pc = 2.0 * (Fj.x * cs + Fj.y * sn);  // d|F|^2 / d amp
        gocc += G * pc * fs * dw;
        gb += G * pc * amp * (-0.25 * g2);
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

extern "C" ds_status ds_simulate_backward(const ds_sim_params *p, const ds_phase_table *t, const double *quats,
                                          int64_t n_orient, const int64_t *offsets, const int32_t *hkl_index,
                                          const double *grad_intensity, double *grad_F2, double *grad_R,
                                          double *grad_recip, void *stream) {
    clear_error();
    DS_REQUIRE(p && t, "ds_simulate_backward: null pointer");
    DS_REQUIRE(n_orient >= 0, "ds_simulate_backward: n_orient < 0");
    DS_REQUIRE(p->k0 > 0 && isfinite(p->k0), "ds_simulate_backward: k0 must be finite and > 0");
    DS_REQUIRE(p->shape_width != 0 && isfinite(p->shape_width), "ds_simulate_backward: bad shape width");
    DS_REQUIRE(p->shape_model >= DS_SHAPE_LINEAR && p->shape_model <= DS_SHAPE_BINARY,
               "ds_simulate_backward: bad shape model");
    DS_REQUIRE(p->precession_mode >= DS_PRECESSION_NONE && p->precession_mode <= DS_PRECESSION_INTEGRAL,
               "ds_simulate_backward: bad precession mode");
    if (n_orient == 0) return DS_OK;
    DS_REQUIRE(quats && offsets && grad_F2 && grad_R && grad_recip, "ds_simulate_backward: null array");
    DS_REQUIRE(t->n_hkl == 0 || (t->hkl && (t->F2 || t->F2d)), "ds_simulate_backward: table arrays missing");
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
    if (c.prec == DS_PRECESSION_INTEGRAL)
        spot_backward_kernel<DS_PRECESSION_INTEGRAL><<<grid, BW_THREADS, 0, s>>>(
            c, quats, offsets, hkl_index, grad_intensity, t->hkl, t->F2, F2d, grad_F2, grad_R, grad_recip);
    else if (c.prec == DS_PRECESSION_LORENTZIAN)
        spot_backward_kernel<DS_PRECESSION_LORENTZIAN><<<grid, BW_THREADS, 0, s>>>(
            c, quats, offsets, hkl_index, grad_intensity, t->hkl, t->F2, F2d, grad_F2, grad_R, grad_recip);
    else
        spot_backward_kernel<DS_PRECESSION_NONE><<<grid, BW_THREADS, 0, s>>>(
            c, quats, offsets, hkl_index, grad_intensity, t->hkl, t->F2, F2d, grad_F2, grad_R, grad_recip);
    return check_launch("spot_backward_kernel");
}

extern "C" size_t ds_structure_factors_backward_scratch_bytes(int64_t n) {
    return n > 0 ? (size_t)n * sizeof(double2) : 0;
}

extern "C" ds_status ds_structure_factors_backward(const ds_atoms *atoms, const int32_t *hkl, const double *g2,
                                                   int64_t n, const double recip[9], const double *grad_F2,
                                                   double *grad_atoms, double *grad_recip, void *scratch,
                                                   size_t scratch_bytes, void *stream) {
    clear_error();
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
    DS_REQUIRE(scratch && scratch_bytes >= ds_structure_factors_backward_scratch_bytes(n),
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
    sf_rows_backward_kernel<<<(unsigned)((n + BW_THREADS - 1) / BW_THREADS), BW_THREADS, 0, s>>>(
        c, *atoms, hkl, g2, grad_F2, F, grad_recip);
    ds_status st = check_launch("sf_rows_backward_kernel");
    if (st) return st;
    const long long n_chunks = (n + SFB_CHUNK - 1) / SFB_CHUNK;
    const long long threads = n_chunks * atoms->n_atoms;
    sf_atoms_backward_kernel<<<(unsigned)((threads + BW_THREADS - 1) / BW_THREADS), BW_THREADS, 0, s>>>(
        c, *atoms, hkl, g2, grad_F2, F, grad_atoms);
    return check_launch("sf_atoms_backward_kernel");
}
