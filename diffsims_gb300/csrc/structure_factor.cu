// A3: kinematical structure factors F_hkl = sum_j f_j(g) occ_j exp(2 pi i h.x_j - B_j g^2 / 4).
//
// Replaces _get_kinematical_structure_factor / get_kinematical_intensities
// (diffsims/utils/sim_utils.py:256-354), its per-site coefficient gather
// (:165-224) and the Lobato / International Tables scattering factors
// (:227-253).  The reference recomputes F for every orientation's selected
// spots (generators/simulation_generator.py:227-234); F depends on hkl and |g|
// only, so here it is one table per phase.
//
// Mixed form: the phase h.x_j is reduced modulo 1 in FP64 (FP64 step #1), the
// rest is FP32 -- sincospi of the reduced phase, f(g), the Debye-Waller factor
// and compensated (two-sum) accumulation, with L lanes per reflection whose
// partial sums meet through warp shuffles.  Reflections whose |F|^2 is small
// against sum_j amplitude_j^2 (strong cancellation, e.g. systematic absences)
// are queued and re-evaluated entirely in FP64, so near-zero |F|^2 come out at
// FP64 size and the reference's 1e-20 * max mask keeps or drops the same spots.
#include <math.h>

#include "common.cuh"

namespace ds {

constexpr int SF_THREADS = 256;
constexpr int SF_MAX_SPECIES = 32;
constexpr int SF_ATOM_CHUNK = 512;
// |F|^2 < SF_KAPPA * sum_j amp_j^2 -> FP64 re-evaluation (about 1% of the
// reflections of a random structure; their FP32 relative error would exceed
// ~2e-6, the rest stay below it).
constexpr float SF_KAPPA = 0.01f;

struct SfConst {
    long long n;
    int n_atoms, n_species, kind, has_hkl_i;
    int g_is_spacing;  // g2 holds |g| (square it) -- the get_kinematical_intensities entry
    int _pad;
    long long mbar_limit;  // polls of the staging wait before it gives up
};

struct SfSmem {
    size_t bar, coeff_f, coeff_d, atoms, occf, bqf, fs, total;
};
__host__ __device__ inline SfSmem sf_smem_layout(int n_species, int chunk) {
    SfSmem L;
    size_t o = 0;
    L.bar = o; o += 16;
    L.coeff_d = o; o += (size_t)n_species * 10 * sizeof(double);
    o = (o + 15) & ~(size_t)15;
    L.coeff_f = o; o += (size_t)n_species * 10 * sizeof(float);
    o = (o + 15) & ~(size_t)15;
    L.atoms = o; o += (size_t)chunk * sizeof(ds_atom);
    L.occf = o; o += (size_t)chunk * sizeof(float);
    L.bqf = o; o += (size_t)chunk * sizeof(float);
    o = (o + 15) & ~(size_t)15;
    L.fs = o; o += (size_t)n_species * SF_THREADS * sizeof(float);
    L.total = o;
    return L;
}

__device__ __forceinline__ void load_hkl(const SfConst &c, const int32_t *hkl_i, const double *hkl_d,
                                         long long j, double &h, double &k, double &l) {
    if (c.has_hkl_i) {
        h = (double)hkl_i[3 * j]; k = (double)hkl_i[3 * j + 1]; l = (double)hkl_i[3 * j + 2];
    } else {
        h = hkl_d[3 * j]; k = hkl_d[3 * j + 1]; l = hkl_d[3 * j + 2];
    }
}

// f_s(g^2) -- the formulas of diffsims/utils/sim_utils.py:249-253.  For the
// two per-family kinds the argument is s^2 = (|g|/2)^2 and the row holds four
// Doyle-Turner pairs plus a constant c0 in slot 8:
//   kinematical  f = c0 - 41.78214 s^2 sum_i a_i exp(-b_i s^2), c0 = Z
//                (diffsims/structure_factor/atomic_scattering_factor.py:55-60)
//   Doyle-Turner f = c0 sum_i a_i exp(-b_i s^2), c0 = 47.87801 / V
//                (diffsims/structure_factor/atomic_scattering_factor.py:111-114)
__device__ __forceinline__ double scatter_f64(const double *cf, int kind, double g2) {
    if (kind == DS_SCATTER_NONE) return 1.0;
    if (kind >= DS_SCATTER_KINEMATICAL) {
        double sum = 0.0;
        for (int i = 0; i < 4; ++i) sum += cf[2 * i] * exp(-cf[2 * i + 1] * g2);
        return kind == DS_SCATTER_KINEMATICAL ? cf[8] - 41.78214 * g2 * sum : cf[8] * sum;
    }
    double f = 0.0;
    for (int i = 0; i < 5; ++i) {
        double a = cf[2 * i], b = cf[2 * i + 1];
        double gb = g2 * b;
        double v = (kind == DS_SCATTER_LOBATO) ? (2.0 + gb) * (1.0 / ((1.0 + gb) * (1.0 + gb)))
                                               : exp(-0.25 * gb);
        f += a * v;
    }
    return f;
}

// Stage coefficients (plain loads, tiny) and prepare the TMA barrier.
__device__ inline void sf_prologue(const SfConst &c, const ds_atoms &A, unsigned char *smem, const SfSmem &L) {
    double *cd = reinterpret_cast<double *>(smem + L.coeff_d);
    float *cf = reinterpret_cast<float *>(smem + L.coeff_f);
    for (int i = threadIdx.x; i < c.n_species * 10; i += blockDim.x) {
        double v = A.coeffs[i];
        cd[i] = v;
        cf[i] = (float)v;
    }
    if (threadIdx.x == 0) mbar_init(reinterpret_cast<uint64_t *>(smem + L.bar), 1);
    __syncthreads();
}

// Copy atoms [start, start+cnt) into shared memory with one TMA bulk copy;
// every thread waits on the barrier (bounded).  Returns false on timeout.
__device__ inline bool sf_stage_chunk(const ds_atoms &A, unsigned char *smem, const SfSmem &L, int start,
                                      int cnt, uint32_t &parity, int32_t *status, bool want_float,
                                      long long limit) {
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L.bar);
    ds_atom *sa = reinterpret_cast<ds_atom *>(smem + L.atoms);
    if (threadIdx.x == 0) {
        uint32_t bytes = (uint32_t)(cnt * sizeof(ds_atom));
        mbar_arrive_expect_tx(bar, bytes);
        tma_bulk_g2s(sa, A.atoms + start, bytes, bar);
    }
    bool ok = mbar_wait_bounded(bar, parity, status, limit);
    parity ^= 1u;
    if (want_float) {
        float *occf = reinterpret_cast<float *>(smem + L.occf);
        float *bqf = reinterpret_cast<float *>(smem + L.bqf);
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
            occf[i] = (float)sa[i].occupancy;
            bqf[i] = (float)(-0.25 * sa[i].B);
        }
    }
    __syncthreads();
    return __syncthreads_and(ok ? 1 : 0) != 0;
}

template <int L>
__global__ void __launch_bounds__(SF_THREADS)
sf_mixed_kernel(SfConst c, ds_atoms A, const int32_t *__restrict__ hkl_i, const double *__restrict__ hkl_d,
                const double *__restrict__ g2in, float *__restrict__ F2, double *__restrict__ F2d,
                double *__restrict__ Fout, int32_t *__restrict__ queue, int32_t *__restrict__ queue_len,
                int32_t *status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int chunk_cap = c.n_atoms < SF_ATOM_CHUNK ? c.n_atoms : SF_ATOM_CHUNK;
    const SfSmem Ls = sf_smem_layout(c.n_species, chunk_cap);
    sf_prologue(c, A, smem, Ls);
    const ds_atom *sa = reinterpret_cast<const ds_atom *>(smem + Ls.atoms);
    const float *occf = reinterpret_cast<const float *>(smem + Ls.occf);
    const float *bqf = reinterpret_cast<const float *>(smem + Ls.bqf);
    float *fs = reinterpret_cast<float *>(smem + Ls.fs);

    const long long j = ((long long)blockIdx.x * SF_THREADS + threadIdx.x) / L;
    const int sub = threadIdx.x % L;
    const bool active = j < c.n;
    double h = 0, k = 0, l = 0, g2 = 0;
    if (active) {
        load_hkl(c, hkl_i, hkl_d, j, h, k, l);
        g2 = g2in[j];
        if (c.g_is_spacing) g2 = g2 * g2;
    }
    const float g2f = (float)g2;
    // f_s(g) in FP64: the Lobato fits sum terms of mixed sign and size, whose
    // cancellation costs FP32 up to ~1e-4 relative.  One evaluation per
    // (reflection, species): the L lanes of a reflection take the species in
    // turn and each value is copied to all L lanes' slots (the per-atom reads
    // stay one slot per thread, free of bank conflicts).  Evaluated on every
    // lane, the FP64 divisions of the fits cost more than the phase work.
    const double *cd = reinterpret_cast<const double *>(smem + Ls.coeff_d);
    {
        const int g0 = threadIdx.x - sub;  // first lane of this reflection's group (same warp)
        for (int s = sub; s < c.n_species; s += L) {
            const float v = (float)scatter_f64(cd + 10 * s, c.kind, g2);
#pragma unroll
            for (int q = 0; q < L; ++q) fs[s * SF_THREADS + g0 + q] = v;
        }
        __syncwarp();
    }

    dd re = {0.f, 0.f}, im = {0.f, 0.f};
    float sumsq = 0.f;
    uint32_t parity = 0;
    for (int start = 0; start < c.n_atoms; start += chunk_cap) {
        int cnt = min(chunk_cap, c.n_atoms - start);
        if (!sf_stage_chunk(A, smem, Ls, start, cnt, parity, status, true, c.mbar_limit)) return;
        if (active) {
            for (int i = sub; i < cnt; i += L) {
                const ds_atom &a = sa[i];
                // FP64 step #1: the phase h.x reduced modulo 1
                double t = fma(h, a.x, fma(k, a.y, l * a.z));
                float tau = 2.f * (float)(t - rint(t));
                float sn, cs;
                sincospif(tau, &sn, &cs);
                float amp = occf[i] * fs[a.species * SF_THREADS + threadIdx.x] * expf(bqf[i] * g2f);
                dd pr = two_sum(re.hi, amp * cs);
                re.hi = pr.hi; re.lo += pr.lo;
                dd pi = two_sum(im.hi, amp * sn);
                im.hi = pi.hi; im.lo += pi.lo;
                sumsq = fmaf(amp, amp, sumsq);
            }
        }
        __syncthreads();
    }
    // combine the L partial sums of a reflection (lanes of one warp)
#pragma unroll
    for (int d = L / 2; d >= 1; d >>= 1) {
        dd ore = {__shfl_xor_sync(FULL_MASK, re.hi, d), __shfl_xor_sync(FULL_MASK, re.lo, d)};
        dd oim = {__shfl_xor_sync(FULL_MASK, im.hi, d), __shfl_xor_sync(FULL_MASK, im.lo, d)};
        float osq = __shfl_xor_sync(FULL_MASK, sumsq, d);
        re = dd_add(re, ore);
        im = dd_add(im, oim);
        sumsq += osq;
    }
    if (!active || sub != 0) return;
    float fre = re.hi + re.lo, fim = im.hi + im.lo;
    float f2 = fre * fre + fim * fim;
    if (f2 < SF_KAPPA * sumsq) {
        int slot = atomicAdd(queue_len, 1);
        queue[slot] = (int32_t)j;
    }
    if (F2) F2[j] = f2;
    if (F2d) F2d[j] = (double)f2;
    if (Fout) { Fout[2 * j] = (double)fre; Fout[2 * j + 1] = (double)fim; }
}

// All-FP64 evaluation of the reflections listed in queue[0 .. *queue_len) (or of
// every reflection when queue is null).  Used for the FP64 form, for the
// get_kinematical_intensities entry and for the mixed form's re-evaluations.
// L lanes share one reflection's atom sum (partial sums meet by shuffles), so
// a short queue still spreads over many SMs' FP64 units.
template <int L>
__global__ void __launch_bounds__(SF_THREADS)
sf_fp64_kernel(SfConst c, ds_atoms A, const int32_t *__restrict__ hkl_i, const double *__restrict__ hkl_d,
               const double *__restrict__ g2in, const double *__restrict__ prefactor, float *__restrict__ F2,
               double *__restrict__ F2d, double *__restrict__ Fout, const int32_t *__restrict__ queue,
               const int32_t *__restrict__ queue_len, int32_t *status) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int PER_BLOCK = SF_THREADS / L;
    const int chunk_cap = c.n_atoms < SF_ATOM_CHUNK ? c.n_atoms : SF_ATOM_CHUNK;
    const SfSmem Ls = sf_smem_layout(c.n_species, chunk_cap);
    const long long n_work = queue ? (long long)(*queue_len) : c.n;
    if ((long long)blockIdx.x * PER_BLOCK >= n_work) return;  // uniform per block
    sf_prologue(c, A, smem, Ls);
    const double *cd = reinterpret_cast<const double *>(smem + Ls.coeff_d);
    const ds_atom *sa = reinterpret_cast<const ds_atom *>(smem + Ls.atoms);
    const int sub = threadIdx.x % L;
    uint32_t parity = 0;  // mbarrier phase, carried across the grid-stride loop

    for (long long base = (long long)blockIdx.x * PER_BLOCK; base < n_work; base += (long long)gridDim.x * PER_BLOCK) {
        const long long w = base + threadIdx.x / L;
        const bool active = w < n_work;
        const long long j = active ? (queue ? (long long)queue[w] : w) : 0;
        double h = 0, k = 0, l = 0, g2 = 0;
        if (active) {
            load_hkl(c, hkl_i, hkl_d, j, h, k, l);
            g2 = g2in[j];
            if (c.g_is_spacing) g2 = g2 * g2;
        }
        double fsp[SF_MAX_SPECIES];
        if constexpr (L == 1) {
            for (int s = 0; s < c.n_species; ++s) fsp[s] = scatter_f64(cd + 10 * s, c.kind, g2);
        } else {
            // one evaluation per (reflection, species): lane sub of the group
            // evaluates species sub, sub + L, ..., and the values are shuffled
            // to the group's lanes (every lane runs every shuffle: n_species
            // and the loop trip counts are uniform)
            constexpr int R = (SF_MAX_SPECIES + L - 1) / L;
            const int g0 = (threadIdx.x & 31) - sub;
            double mine[R];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int s = sub + r * L;
                mine[r] = s < c.n_species ? scatter_f64(cd + 10 * s, c.kind, g2) : 0.0;
            }
#pragma unroll
            for (int s = 0; s < SF_MAX_SPECIES; ++s)
                if (s < c.n_species) fsp[s] = __shfl_sync(FULL_MASK, mine[s / L], g0 + s % L);
        }
        double re = 0.0, im = 0.0;
        // amplitude of the previous atom: consecutive atoms with the same
        // species, occupancy and B (the positions of one orbit) reuse it
        double amp = 0.0, occ_prev = 0.0, B_prev = 0.0;
        int sp_prev = -1;
        for (int start = 0; start < c.n_atoms; start += chunk_cap) {
            int cnt = min(chunk_cap, c.n_atoms - start);
            if (!sf_stage_chunk(A, smem, Ls, start, cnt, parity, status, false, c.mbar_limit)) return;
            if (active) {
                for (int i = sub; i < cnt; i += L) {
                    const ds_atom &a = sa[i];
                    double t = h * a.x + k * a.y + l * a.z;
                    double r = t - rint(t);
                    double sn, cs;
                    sincospi(2.0 * r, &sn, &cs);
                    if (a.species != sp_prev || a.occupancy != occ_prev || a.B != B_prev) {
                        amp = fsp[a.species] * a.occupancy * exp(-0.25 * g2 * a.B);
                        sp_prev = a.species; occ_prev = a.occupancy; B_prev = a.B;
                    }
                    re = fma(amp, cs, re);
                    im = fma(amp, sn, im);
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int d = L / 2; d >= 1; d >>= 1) {
            re += __shfl_xor_sync(FULL_MASK, re, d);
            im += __shfl_xor_sync(FULL_MASK, im, d);
        }
        if (active && sub == 0) {
            double f2 = re * re + im * im;
            if (prefactor) f2 *= prefactor[j];
            if (F2) F2[j] = (float)f2;
            if (F2d) F2d[j] = f2;
            if (Fout) { Fout[2 * j] = re; Fout[2 * j + 1] = im; }
        }
    }
}

static ds_status validate_atoms(const ds_atoms *A) {
    DS_REQUIRE(A && A->atoms && A->coeffs, "structure factors: null atoms");
    DS_REQUIRE(A->n_atoms >= 1, "structure factors: n_atoms must be >= 1");
    DS_REQUIRE(A->n_species >= 1 && A->n_species <= SF_MAX_SPECIES,
               "structure factors: n_species must be in [1, 32]");
    DS_REQUIRE(A->kind >= DS_SCATTER_LOBATO && A->kind <= DS_SCATTER_NONE, "structure factors: bad kind");
    DS_REQUIRE(((uintptr_t)A->atoms & 15) == 0, "structure factors: atoms must be 16-byte aligned");
    return DS_OK;
}

template <int L>
static ds_status launch_fp64_l(const SfConst &c, const ds_atoms &A, const int32_t *hkl_i, const double *hkl_d,
                               const double *g2, const double *pref, float *F2, double *F2d, double *F,
                               const int32_t *queue, const int32_t *queue_len, long long max_work,
                               int32_t *status, cudaStream_t s) {
    int chunk = c.n_atoms < SF_ATOM_CHUNK ? c.n_atoms : SF_ATOM_CHUNK;
    SfSmem Ls = sf_smem_layout(c.n_species, chunk);
    DS_CUDA_TRY(cudaFuncSetAttribute(sf_fp64_kernel<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Ls.total));
    long long blocks = (max_work * L + SF_THREADS - 1) / SF_THREADS;
    if (blocks > 8192) blocks = 8192;
    sf_fp64_kernel<L><<<(unsigned)blocks, SF_THREADS, Ls.total, s>>>(c, A, hkl_i, hkl_d, g2, pref, F2, F2d, F, queue,
                                                                    queue_len, status);
    return check_launch("sf_fp64_kernel");
}

// L lanes per reflection: whole warps for short lists and many atoms, one lane
// per reflection when the reflections alone fill the GPU.
static ds_status launch_fp64(const SfConst &c, const ds_atoms &A, const int32_t *hkl_i, const double *hkl_d,
                             const double *g2, const double *pref, float *F2, double *F2d, double *F,
                             const int32_t *queue, const int32_t *queue_len, long long max_work,
                             int32_t *status, cudaStream_t s) {
    if (max_work <= 0) return DS_OK;
    const long long want = 152ll * 2048;
    if (queue) {  // typically ~1% of the table: a warp per reflection
        if (c.n_atoms >= 32) return launch_fp64_l<32>(c, A, hkl_i, hkl_d, g2, pref, F2, F2d, F, queue, queue_len, max_work, status, s);
        return launch_fp64_l<8>(c, A, hkl_i, hkl_d, g2, pref, F2, F2d, F, queue, queue_len, max_work, status, s);
    }
    if (max_work >= want || c.n_atoms < 8)
        return launch_fp64_l<1>(c, A, hkl_i, hkl_d, g2, pref, F2, F2d, F, queue, queue_len, max_work, status, s);
    if (max_work * 4 >= want || c.n_atoms < 32)
        return launch_fp64_l<4>(c, A, hkl_i, hkl_d, g2, pref, F2, F2d, F, queue, queue_len, max_work, status, s);
    return launch_fp64_l<32>(c, A, hkl_i, hkl_d, g2, pref, F2, F2d, F, queue, queue_len, max_work, status, s);
}

template <int L>
static ds_status launch_mixed(const SfConst &c, const ds_atoms &A, const int32_t *hkl_i, const double *hkl_d,
                              const double *g2, float *F2, double *F2d, double *F, int32_t *queue,
                              int32_t *queue_len, int32_t *status, cudaStream_t s) {
    int chunk = c.n_atoms < SF_ATOM_CHUNK ? c.n_atoms : SF_ATOM_CHUNK;
    SfSmem Ls = sf_smem_layout(c.n_species, chunk);
    DS_CUDA_TRY(cudaFuncSetAttribute(sf_mixed_kernel<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Ls.total));
    long long blocks = (c.n * L + SF_THREADS - 1) / SF_THREADS;
    sf_mixed_kernel<L><<<(unsigned)blocks, SF_THREADS, Ls.total, s>>>(c, A, hkl_i, hkl_d, g2, F2, F2d, F, queue,
                                                                     queue_len, status);
    return check_launch("sf_mixed_kernel");
}

}  // namespace ds

using namespace ds;

extern "C" size_t ds_structure_factor_scratch_bytes(int64_t n_hkl, int32_t /*n_atoms*/) {
    return (size_t)(n_hkl + 64) * sizeof(int32_t);
}

extern "C" ds_status ds_structure_factors(const ds_atoms *atoms, const int32_t *hkl_i, const double *hkl_d,
                                          const double *g2, int64_t n, int32_t form, float *F2, double *F2d,
                                          double *F, void *scratch, size_t scratch_bytes, int32_t *status,
                                          void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_structure_factors");
    ds_status st = validate_atoms(atoms);
    if (st) return st;
    DS_REQUIRE((hkl_i != nullptr) != (hkl_d != nullptr), "ds_structure_factors: give exactly one of hkl_i, hkl_d");
    DS_REQUIRE(g2 && status, "ds_structure_factors: null pointer");
    DS_REQUIRE(n >= 0, "ds_structure_factors: n < 0");
    DS_REQUIRE(form == DS_FORM_MIXED || form == DS_FORM_FP64, "ds_structure_factors: bad form");
    if (n == 0) return DS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    SfConst c{n, atoms->n_atoms, atoms->n_species, atoms->kind, hkl_i != nullptr, 0, 0, wait_limit_mbarrier()};
    if (form == DS_FORM_FP64)
        return launch_fp64(c, *atoms, hkl_i, hkl_d, g2, nullptr, F2, F2d, F, nullptr, nullptr, n, status, s);
    DS_REQUIRE(scratch && scratch_bytes >= ds_structure_factor_scratch_bytes(n, atoms->n_atoms),
               "ds_structure_factors: scratch too small");
    int32_t *queue_len = reinterpret_cast<int32_t *>(scratch);
    int32_t *queue = queue_len + 64;
    DS_CUDA_TRY(cudaMemsetAsync(queue_len, 0, sizeof(int32_t), s));
    // lanes per reflection: spread the atom sum over more lanes when there are
    // too few reflections to fill the GPU (152 SMs x 2048 threads)
    long long want_threads = 152ll * 2048;
    if (n >= want_threads || atoms->n_atoms < 8) st = launch_mixed<1>(c, *atoms, hkl_i, hkl_d, g2, F2, F2d, F, queue, queue_len, status, s);
    else if (n * 2 >= want_threads || atoms->n_atoms < 32) st = launch_mixed<2>(c, *atoms, hkl_i, hkl_d, g2, F2, F2d, F, queue, queue_len, status, s);
    else if (n * 4 >= want_threads) st = launch_mixed<4>(c, *atoms, hkl_i, hkl_d, g2, F2, F2d, F, queue, queue_len, status, s);
    else st = launch_mixed<8>(c, *atoms, hkl_i, hkl_d, g2, F2, F2d, F, queue, queue_len, status, s);
    if (st) return st;
    return launch_fp64(c, *atoms, hkl_i, hkl_d, g2, nullptr, F2, F2d, F, queue, queue_len, n, status, s);
}

extern "C" ds_status ds_family_structure_factors(const ds_atoms *atoms, const double *hkl_d,
                                                 const double *scattering_parameter, int64_t n, double *F,
                                                 int32_t *status, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_family_structure_factors");
    DS_REQUIRE(atoms && atoms->atoms && atoms->coeffs, "ds_family_structure_factors: null atoms");
    DS_REQUIRE(atoms->n_atoms >= 1, "ds_family_structure_factors: n_atoms must be >= 1");
    DS_REQUIRE(atoms->n_species >= 1 && atoms->n_species <= SF_MAX_SPECIES,
               "ds_family_structure_factors: n_species must be in [1, 32]");
    DS_REQUIRE(atoms->kind == DS_SCATTER_KINEMATICAL || atoms->kind == DS_SCATTER_DOYLETURNER,
               "ds_family_structure_factors: kind must be DS_SCATTER_KINEMATICAL or DS_SCATTER_DOYLETURNER");
    DS_REQUIRE(((uintptr_t)atoms->atoms & 15) == 0, "ds_family_structure_factors: atoms must be 16-byte aligned");
    DS_REQUIRE(n >= 0, "ds_family_structure_factors: n < 0");
    if (n == 0) return DS_OK;
    DS_REQUIRE(hkl_d && scattering_parameter && F && status, "ds_family_structure_factors: null pointer");
    // g_is_spacing squares the per-reflection input: the kernel sees s^2
    SfConst c{n, atoms->n_atoms, atoms->n_species, atoms->kind, 0, 1, 0, wait_limit_mbarrier()};
    return launch_fp64(c, *atoms, nullptr, hkl_d, scattering_parameter, nullptr, nullptr, nullptr, F, nullptr,
                       nullptr, n, status, (cudaStream_t)stream);
}

extern "C" ds_status ds_kinematical_intensities(const ds_atoms *atoms, const double *hkl_d, const double *g_spacing,
                                                const double *prefactor, int64_t n, double *out, void * /*scratch*/,
                                                size_t /*scratch_bytes*/, int32_t *status, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_kinematical_intensities");
    ds_status st = validate_atoms(atoms);
    if (st) return st;
    DS_REQUIRE(hkl_d && g_spacing && out && status, "ds_kinematical_intensities: null pointer");
    DS_REQUIRE(n >= 0, "ds_kinematical_intensities: n < 0");
    if (n == 0) return DS_OK;
    SfConst c{n, atoms->n_atoms, atoms->n_species, atoms->kind, 0, 1, 0, wait_limit_mbarrier()};
    return launch_fp64(c, *atoms, nullptr, hkl_d, g_spacing, prefactor, nullptr, out, nullptr, nullptr, nullptr, n,
                       status, (cudaStream_t)stream);
}
