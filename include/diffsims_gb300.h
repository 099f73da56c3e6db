/*
 * diffsims_gb300 -- C ABI of the GB300 (sm_103a) kinematical spot-pattern path.
 *
 * Every device buffer is owned by the caller (plain device pointers and
 * sizes; no torch types).  Every compute call is asynchronous on the given
 * CUDA stream; a host-side status (ds_status) reports argument and launch
 * errors immediately, a device status word (int32, caller-owned) reports
 * data-dependent conditions (output capacity, bounded-wait timeouts) once the
 * stream is synchronised.  The library never allocates device memory: the
 * callers size scratch with the *_scratch_bytes queries.
 *
 * The reference (diffsims 0.7.x) is pure Python; the entries below replace
 * the numpy arithmetic behind its public calls.  Citations are paths inside
 * that project.
 */
#ifndef DIFFSIMS_GB300_H
#define DIFFSIMS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t ds_status;
enum {
    DS_OK = 0,
    DS_ERR_INVALID_ARGUMENT = 1,
    DS_ERR_CUDA = 2,
    DS_ERR_CAPACITY = 4,      /* device word bit: output capacity exceeded   */
    DS_ERR_TIMEOUT = 8,       /* device word bit: a bounded wait gave up     */
    DS_ERR_UNSUPPORTED = 16,
    DS_ERR_NONFINITE = 32,    /* device word bit: non-finite input met       */
    DS_ERR_BOUNDS = 64        /* device word bit, bounds-checked builds only
                                 (-DDS_DEBUG_BOUNDS): an index check failed
                                 and the access was skipped                  */
};

/* arithmetic form of a call */
enum { DS_FORM_MIXED = 0, /* FP32 bulk, FP64 phase reduction + FP64 s near the cutoff */
       DS_FORM_FP64 = 1   /* plain all-FP64 comparator                              */ };

/* scattering factor parameterisation (diffsims/utils/sim_utils.py:139-162,227-253);
 * the last two serve ds_family_structure_factors only
 * (diffsims/structure_factor/atomic_scattering_factor.py:27-124) */
enum { DS_SCATTER_LOBATO = 0, DS_SCATTER_XTABLES = 1, DS_SCATTER_NONE = 2,
       DS_SCATTER_KINEMATICAL = 3, DS_SCATTER_DOYLETURNER = 4 };

/* rel-rod shape models (diffsims/utils/shape_factor_models.py) */
enum { DS_SHAPE_LINEAR = 0, DS_SHAPE_ATANC = 1, DS_SHAPE_SINC = 2, DS_SHAPE_SIN2C = 3,
       DS_SHAPE_LORENTZIAN = 4, DS_SHAPE_BINARY = 5 };

/* candidate screen of ds_simulate: a test per (orientation, row); per-
 * (orientation, hkl line) intervals; or bricks -- the rows grouped into
 * compact blocks of hkl, each block tested once per orientation and its rows
 * only where the block passes (the same per-row test, so the same rows are
 * kept).  All keep a superset of the selected spots and the exact selection
 * follows, so the results are identical.  AUTO: rows (the fastest measured
 * on the large single-phase workload). */
enum { DS_SCREEN_AUTO = 0, DS_SCREEN_ROWS = 1, DS_SCREEN_LINES = 2, DS_SCREEN_BRICKS = 3 };

/* precession handling (diffsims/generators/simulation_generator.py:363-411) */
enum { DS_PRECESSION_NONE = 0,
       DS_PRECESSION_LORENTZIAN = 1, /* approximate_precession=True: lorentzian_precession */
       DS_PRECESSION_INTEGRAL = 2    /* approximate_precession=False: rotation average     */ };

/* ---------------------------------------------------------------- A1 ---- */
/* Per-axis hkl box half-widths: first n with 1/|n e_i| <= min_dspacing.
 * Replaces orix _get_highest_hkl as called at
 * diffsims/crystallography/reciprocal_lattice_vector.py:1131-1133 (rule stated at
 * diffsims/crystallography/get_hkl.py:49-57).  Host only.
 * recip: rows a*, b*, c* (1/Angstrom, no 2 pi) in the x||a, z||c* frame. */
ds_status ds_box_extent(const double recip[9], double min_dspacing, int32_t hmax_out[3]);

/* Scratch bytes for ds_enumerate_hkl with this box. */
size_t ds_enumerate_scratch_bytes(const int32_t hmax[3]);

/* Ordered hkl set of ReciprocalLatticeVector.from_min_dspacing
 * (diffsims/crystallography/reciprocal_lattice_vector.py:1131-1141): the box
 * in descending (h,k,l) order without 000, kept where 1/|g| >= min_dspacing,
 * followed by n_zero rows of 000 (from_min_dspacing's include_zero_vector and
 * the second 000 of generators/simulation_generator.py:351-353).
 * hkl_out: capacity x 3 int32; g2_out: capacity doubles (|g|^2); count_out:
 * one int64 (device) = rows written.  capacity must be >= box size + n_zero. */
ds_status ds_enumerate_hkl(const double recip[9], const int32_t hmax[3], double min_dspacing,
                           int32_t n_zero, int32_t *hkl_out, double *g2_out, int64_t capacity,
                           int64_t *count_out, void *scratch, size_t scratch_bytes,
                           int32_t *status, void *stream);

/* get_points_in_sphere (diffsims/utils/sim_utils.py:436-474), the candidate
 * set of the legacy DiffractionGenerator.calculate_ed_data
 * (diffsims/generators/diffraction_generator.py:238-241): the box
 * [-H..H] x [-K..K] x [-L..L] in itertools.product order (h slowest, l
 * fastest, ascending), 000 included where it falls, kept where |g| < radius
 * (|g|^2 in the fixed operation order of ds_enumerate_hkl, then sqrt).
 * hmax: floor(radius / |a*|), floor(radius / |b*|), floor(radius / |c*|);
 * capacity >= box size; scratch sized by ds_enumerate_scratch_bytes. */
ds_status ds_enumerate_sphere(const double recip[9], const int32_t hmax[3], double radius,
                              int32_t *hkl_out, double *g2_out, int64_t capacity, int64_t *count_out,
                              void *scratch, size_t scratch_bytes, int32_t *status, void *stream);

/* ---------------------------------------------------------------- A3 ---- */
/* One atom of a phase: 48-byte record (a multiple of 16 so the atom table can
 * be staged into shared memory with 1-D TMA bulk copies). */
typedef struct {
    double x, y, z;           /* fractional coordinates                        */
    double occupancy;
    double B;                 /* Debye-Waller B (Angstrom^2)                   */
    int32_t species;          /* row of ds_atoms.coeffs                        */
    int32_t _pad;
} ds_atom;

/* One phase's atoms (device arrays; both 16-byte aligned). */
typedef struct {
    int32_t n_atoms;
    int32_t n_species;
    const ds_atom *atoms;     /* n_atoms records                                 */
    const double *coeffs;     /* n_species x 10: a1,b1,...,a5,b5 (zeros = unknown element) */
    int32_t kind;             /* DS_SCATTER_*                                    */
    int32_t _pad;
} ds_atoms;

size_t ds_structure_factor_scratch_bytes(int64_t n_hkl, int32_t n_atoms);

/* Structure factors of n reflections: F = sum_j f_j occ_j exp(2 pi i h.x_j - B_j g^2/4)
 * (diffsims/utils/sim_utils.py:256-304).  Exactly one of hkl_i (int32 n x 3) and
 * hkl_d (double n x 3, non-integer indices allowed) is non-null.  g2: |g|^2 per
 * reflection.  Outputs (any may be null): F2 (float |F|^2), F2d (double |F|^2),
 * F (double re, im pairs).  form DS_FORM_MIXED: FP64 phase reduction frac(h.x),
 * FP32 sincospi / scattering factors / Debye-Waller with compensated sums, and
 * an FP64 re-evaluation of the reflections whose |F|^2 is small against
 * sum_j |amplitude_j|^2; DS_FORM_FP64: all FP64. */
ds_status ds_structure_factors(const ds_atoms *atoms, const int32_t *hkl_i, const double *hkl_d,
                               const double *g2, int64_t n, int32_t form, float *F2, double *F2d,
                               double *F, void *scratch, size_t scratch_bytes, int32_t *status,
                               void *stream);

/* Structure factors of lattice-plane families, batched over n reflections:
 * get_kinematical_structure_factor and get_doyleturner_structure_factor
 * (diffsims/structure_factor/structure_factor.py:55-185) before their scalar
 * epilogues.  F[2i], F[2i+1] = sum_j f_j(s_i) occ_j exp(-B_j s_i^2) (cos, +sin)
 * (2 pi h_i.x_j), all FP64 with the phase reduced modulo 1 first; the
 * reference's sign is exp(-2 pi i h.x), i.e. the conjugate.  atoms->kind is
 * DS_SCATTER_KINEMATICAL or DS_SCATTER_DOYLETURNER; each coeffs row holds
 * a1,b1,...,a4,b4 (Doyle-Turner, 1/Angstrom^2), then c0 (Z, or 47.87801 / unit
 * cell volume) and 0; each record's B holds 4 x Bisoequiv (the kernel's
 * Debye-Waller term is exp(-B s^2 / 4) in s = scattering_parameter).  The atom
 * list is the expanded orbit (the caller applies the space group). */
ds_status ds_family_structure_factors(const ds_atoms *atoms, const double *hkl_d,
                                      const double *scattering_parameter, int64_t n, double *F,
                                      int32_t *status, void *stream);

/* get_kinematical_intensities (diffsims/utils/sim_utils.py:307-354):
 * out[i] = prefactor[i] * |F_i|^2 with |g| given (not derived from the lattice).
 * prefactor may be null (1).  Computed in FP64. */
ds_status ds_kinematical_intensities(const ds_atoms *atoms, const double *hkl_d, const double *g_spacing,
                                     const double *prefactor, int64_t n, double *out, void *scratch,
                                     size_t scratch_bytes, int32_t *status, void *stream);

/* ------------------------------------------------------------- A4-A7 ---- */
typedef struct {
    double k0;                   /* 1 / wavelength (1/Angstrom)                     */
    double max_excitation_error; /* selection cut-off                               */
    double shape_width;          /* shape_factor_width or max_excitation_error      */
    double precession_angle;     /* radians (>= 0)                                  */
    double minimum_intensity;    /* mask: keep I > max_pattern(I) * this            */
    double minima_number;        /* sinc / sin2c / atanc parameter (default 5)      */
    int32_t shape_model;         /* DS_SHAPE_*                                      */
    int32_t precession_mode;     /* DS_PRECESSION_*                                 */
    int32_t form;                /* DS_FORM_*                                       */
    int32_t orient_tile;         /* orientations per CTA (0 = library choice)       */
    int32_t stage_cap;           /* staged candidates per CTA (0 = library choice)  */
    int32_t screen;              /* DS_SCREEN_* (0 = library choice)                */
    int32_t refine_parts;        /* reflections per work unit of the refine and
                                    write passes: each orientation's candidate
                                    bitmap is cut into this many word ranges
                                    (1, 2, 4 or 8; 0 = library choice)            */
    int32_t _reserved;           /* 0                                               */
} ds_sim_params;

/* One phase's candidate table (device arrays of n_hkl rows, in reference order). */
typedef struct {
    int64_t n_hkl;
    const int32_t *hkl;          /* n_hkl x 3                                      */
    const double *g2;            /* n_hkl |g|^2                                    */
    const float *F2;             /* n_hkl |F|^2 (mixed form)                       */
    const double *F2d;           /* n_hkl |F|^2 (FP64 form; may be null for mixed) */
    double recip[9];             /* rows a*, b*, c*: g = hkl @ recip               */
    int32_t hmax[3];             /* max |h|, |k|, |l| in the table                 */
    int32_t _pad;
} ds_phase_table;

/* Output spots in CSR form (device-addressable arrays: device memory, or
 * page-locked host memory that ds_host_mapped reports as mapped, in which
 * case the kernel's own stores carry the spots to the host). */
typedef struct {
    int64_t *offsets;            /* n_orient + 1                                   */
    int32_t *hkl_index;          /* capacity: row of the candidate table           */
    float *xyzi;                 /* capacity x 4: beam-frame x, y, z, intensity    */
    int64_t capacity;
    int64_t *total;              /* one int64: spots of the call (may exceed capacity) */
    double *excitation_error;    /* capacity, optional (null): s of every spot      */
    int32_t hkl_index_bytes;     /* 0 or 4: int32 rows; 2: uint16 rows (ds_simulate
                                    with tables of at most 65536 rows only; hkl_index
                                    then points at capacity uint16 values)        */
    int32_t _reserved;           /* 0 */
} ds_spots;

size_t ds_simulate_scratch_bytes(const ds_sim_params *p, const ds_phase_table *t, int64_t n_orient);

/* The per-orientation loop of SimulationGenerator.calculate_diffraction2d
 * (diffsims/generators/simulation_generator.py:211-241) with
 * get_intersecting_reflections (:319-412): rotate the table into the beam frame
 * (R(q)^T g), excitation error, selection, shape factor, I = sf |F|^2, the
 * minimum-intensity mask, ordered compaction into CSR.
 * quats: n_orient x 4 doubles (w, x, y, z) -- active rotation of the crystal.
 * On capacity overflow *total still gets the exact size, offsets are exact,
 * rows beyond capacity are not written and DS_ERR_CAPACITY is or-ed into
 * *status: re-run with capacity >= *total.  out->hkl_index_bytes = 2 writes
 * the rows as uint16 (tables of at most 65536 rows): 18 instead of 20 bytes
 * per spot for results that travel to the host. */
ds_status ds_simulate(const ds_sim_params *p, const ds_phase_table *t, const double *quats,
                      int64_t n_orient, ds_spots *out, void *scratch, size_t scratch_bytes,
                      int32_t *status, void *stream);

/* One phase of a batched call: its candidate table and its orientations. */
typedef struct {
    ds_phase_table table;
    const double *quats;         /* n_orient x 4 (device)                           */
    int64_t n_orient;
} ds_batch_phase;

size_t ds_simulate_batch_scratch_bytes(const ds_sim_params *p, const ds_batch_phase *phases,
                                       int32_t n_phases);
/* Orientations per tile the batched launch would use (0 on bad arguments). */
int32_t ds_simulate_batch_tile(const ds_sim_params *p, const ds_batch_phase *phases, int32_t n_phases);

/* No counterpart in the reference (calculate_diffraction2d loops over phases,
 * diffsims/generators/simulation_generator.py:198-241): ds_simulate for up to 96
 * phases in ONE persistent launch (plus one small prep launch per phase).
 * Tiles of up to p->orient_tile orientations (0: library choice; at most 32,
 * 16 with the precession average, 8 for the FP64 form; phases whose tables
 * would overflow shared memory use smaller tiles) run phase after phase from
 * one tile ticket.  The output is
 * one CSR over all phases' orientations in phase order (offsets:
 * sum n_orient + 1); hkl_index holds rows of each spot's own phase table.
 * Capacity rules as ds_simulate.  Graph-capturable: the phase descriptors are
 * a kernel parameter. */
ds_status ds_simulate_batch(const ds_sim_params *p, const ds_batch_phase *phases, int32_t n_phases,
                            ds_spots *out, void *scratch, size_t scratch_bytes, int32_t *status,
                            void *stream);

/* No counterpart in the reference.  ds_simulate for callers that cannot
 * allocate device memory at all (e.g. a real-time loop that must not enter the
 * CUDA allocator, or a host whose memory manager owns all device memory):
 * the scratch of ds_simulate comes from a static 64 MiB device array in the
 * library instead of a caller buffer; inputs and outputs are still the
 * caller's.  Sizes whose scratch does not fit (after shrinking the candidate
 * staging) return DS_ERR_INVALID_ARGUMENT.  All calls share the array: calls
 * that overlap on the GPU race (one stream is safe).  Every call looks the
 * array's address up (cudaGetSymbolAddress, the caller's device current), so
 * a device reset between calls is safe; the first call on a device loads the
 * library's device code: make it before any stream capture.  A problem the
 * library cannot plan returns the plan's own status and message.  Allocates
 * nothing. */
ds_status ds_simulate_noalloc(const ds_sim_params *p, const ds_phase_table *t, const double *quats,
                              int64_t n_orient, ds_spots *out, int32_t *status, void *stream);

/* Custom shape factors: the last step of calculate_diffraction2d with a
 * shape-factor function of the caller's
 * (diffsims/generators/simulation_generator.py:117-120,387-411), which
 * cannot run in a kernel.  The spots come from ds_simulate with the model
 * switched off (DS_SHAPE_BINARY, minimum_intensity < 0: every selected row,
 * its excitation error requested); the caller evaluates its function on
 * them; this call finishes each pattern: I = shape_factors[k] * F2[row]
 * (FP64 product), keeps I > max(pattern I) * minimum_intensity (:237-240)
 * and compacts the kept spots in order into out (x, y, z copied, I
 * replaced).  offsets_in / hkl_index_in / xyzi_in: the first call's CSR;
 * shape_factors: one per input spot; F2: the table's |F|^2 (mixed form).
 * Capacity overflow as ds_simulate.  scratch: ds_apply_shape_factors_scratch_bytes. */
size_t ds_apply_shape_factors_scratch_bytes(int64_t n_patterns);
ds_status ds_apply_shape_factors(const int64_t *offsets_in, const int32_t *hkl_index_in, const float *xyzi_in,
                                 const double *shape_factors, const float *F2, int64_t n_patterns,
                                 double minimum_intensity, ds_spots *out, void *scratch, size_t scratch_bytes,
                                 int32_t *status, void *stream);

/* ------------------------------------------------------------------------ */
/* Detector images of spot patterns.  Replaces Simulation2D.get_diffraction_pattern
 * (diffsims/simulations/simulation2d.py:357-442) with
 * get_pattern_from_pixel_coordinates_and_intensities and _subpixel_gaussian
 * (diffsims/pattern/detector_functions.py:251-359), for many patterns per call. */
typedef struct {
    int32_t height, width;       /* detector shape (rows, columns), pixels           */
    int32_t mirrored;            /* 1: mirror across the x axis                      */
    int32_t fast;                /* 1: truncate to whole pixels, last write wins,
                                    Gaussian filter (mode reflect); 0: sub-pixel
                                    boxed Gaussians (_subpixel_gaussian)             */
    int32_t normalize;           /* 1: divide by the image maximum                   */
    int32_t _pad;
    double sigma;                /* Gaussian standard deviation, pixels              */
    double calibration;          /* 1/Angstrom per pixel                             */
    double center_x, center_y;   /* direct-beam position, pixels                     */
    double in_plane_angle;       /* degrees                                          */
    double clip_threshold;       /* fast == 0: value below which a spot's box ends   */
    double truncate;             /* fast == 1: filter radius int(truncate*sigma+0.5) */
    double pixel_snap;           /* >= 0: positions within this of a whole pixel are
                                    moved onto it (0: the reference's exact rule)    */
} ds_raster_params;

/* Device scratch ds_rasterize needs for patterns of up to max_spots spots
 * (0 when the per-pattern work fits in shared memory). */
size_t ds_rasterize_scratch_bytes(const ds_raster_params *p, int64_t max_spots);

/* n_patterns images of height x width float32 into out (pattern-major).
 * offsets: n_patterns + 1 int64 (absolute rows of xyzi), xyzi: rows of
 * (x, y, z, intensity) float32 in the beam frame (the ds_spots layout).
 * max_spots: an upper bound on offsets[i+1] - offsets[i]; a pattern above it
 * is left unwritten and DS_ERR_CAPACITY is or-ed into *status. */
ds_status ds_rasterize(const ds_raster_params *p, const int64_t *offsets, const float *xyzi,
                       int64_t n_patterns, int64_t max_spots, float *out, void *scratch,
                       size_t scratch_bytes, int32_t *status, void *stream);

/* ------------------------------------------------------------------------ */
/* Padded polar templates: Simulation2D.polar_flatten_simulations
 * (diffsims/simulations/simulation2d.py:313-355) for n_patterns CSR patterns
 * (offsets absolute rows of xyzi).  Outputs n_patterns x max_spots doubles
 * each, zero padded: r = |(x, y)|, theta = atan2(y, x), intensity.  With both
 * axes (sorted ascending), r and theta become the indices of the closest axis
 * entries (get_closest, simulation2d.py:767-781) and spots whose index reaches
 * the last entry of either axis are dropped (the kept ones stay in order). */
ds_status ds_polar_flatten(const int64_t *offsets, const float *xyzi, int64_t n_patterns, int64_t max_spots,
                           const double *radial_axes, int64_t n_radial, const double *azimuthal_axes,
                           int64_t n_azimuthal, double *r_out, double *theta_out, double *intensity_out,
                           void *stream);

/* ds_polar_flatten with r and theta computed in FP32 (sqrtf of x x + y y
 * rounded in FP32, atan2f) and the axes given as float and searched in FP32;
 * the outputs are the same float64 arrays.  r and theta agree with the FP64
 * entry to ~2e-7 relative (the order of the float32 spot positions' own
 * rounding); closest-axis indices can differ only for values that close to a
 * decision boundary.  Bound by its bytes instead of the FP64 pipe.  No
 * counterpart in the reference beyond ds_polar_flatten's. */
ds_status ds_polar_flatten_f32(const int64_t *offsets, const float *xyzi, int64_t n_patterns, int64_t max_spots,
                               const float *radial_axes, int64_t n_radial, const float *azimuthal_axes,
                               int64_t n_azimuthal, double *r_out, double *theta_out, double *intensity_out,
                               void *stream);

/* ------------------------------------------------------------------------ */
/* Adjoint of the spot intensities I = shf(s, r) |F_hkl|^2 (no counterpart in
 * the reference, which is not differentiable).  After a ds_simulate call with
 * the same p, t and quats, whose output had n_spots spots:
 * grad_intensity[j] = dL/dI for every output spot j.  Accumulates (+=)
 * dL/d|F|^2 per table row into grad_F2 (n_hkl doubles) and dL/dB* into
 * grad_recip (9 doubles, B* = t->recip, rows a*, b*, c*); writes dL/dq
 * (n_orient x 4 doubles, through the normalisation of q).  Selection is
 * piecewise constant and not differentiated.  Scratch (the rotation average's
 * per-spot partials) from ds_simulate_backward_scratch_bytes. */
size_t ds_simulate_backward_scratch_bytes(const ds_sim_params *p, int64_t n_spots, int64_t n_orient);
ds_status ds_simulate_backward(const ds_sim_params *p, const ds_phase_table *t, const double *quats,
                               int64_t n_orient, const int64_t *offsets, const int32_t *hkl_index,
                               int64_t n_spots, const double *grad_intensity, double *grad_F2,
                               double *grad_quats, double *grad_recip, void *scratch, size_t scratch_bytes,
                               int32_t *status, void *stream);

/* Orientation corrections (no counterpart in the reference): quats_out = q0 (x)
 * exp(rotvec), the Hamilton product with the unit quaternion of each rotation
 * vector (n x 3 doubles, angle = length in radians); and its adjoint,
 * grad_rotvec = dL/drotvec from grad_quats = dL/dquats_out. */
ds_status ds_axis_angle_compose(const double *q0, const double *rotvec, int64_t n, double *quats_out,
                                void *stream);
ds_status ds_axis_angle_compose_backward(const double *q0, const double *rotvec, int64_t n,
                                         const double *grad_quats, double *grad_rotvec, void *stream);

size_t ds_structure_factors_backward_scratch_bytes(int64_t n, int32_t n_species);

/* Adjoint of ds_structure_factors: from dL/d|F|^2 per row, accumulates (+=)
 * dL/d(x, y, z, occupancy, B) per atom into grad_atoms (n_atoms x 5 doubles)
 * and dL/dB* through |g|^2 (scattering factors, Debye-Waller) into grad_recip.
 * recip: host array, the rows' reciprocal basis.  F is recomputed (phase
 * reduced in FP64, FP32 products, FP64 sums). */
ds_status ds_structure_factors_backward(const ds_atoms *atoms, const int32_t *hkl, const double *g2, int64_t n,
                                        const double recip[9], const double *grad_F2, double *grad_atoms,
                                        double *grad_recip, void *scratch, size_t scratch_bytes, void *stream);

/* ------------------------------------------------------------------------ */
/* FP32 FMA throughput probe (no counterpart in the reference): blocks x 256
 * threads, each 8 chains x 16 x iters fused multiply-adds; out holds
 * blocks*256 floats.  FLOPs = blocks * 256 * iters * 256.  Used to measure the
 * FP32 roofline denominator. */
ds_status ds_probe_fp32_fma(int64_t iters, int32_t blocks, float *out, void *stream);

/* Bounded device waits (no counterpart in the reference, which has no device
 * code on this path).  Every spin of the kernels gives up after a number of
 * polls, sets DS_ERR_TIMEOUT in the status word and returns: the decoupled
 * look-back's wait for an earlier tile (default 2^24 polls with backoff) and
 * the structure-factor kernels' wait for a staging copy (default 2^22 polls;
 * after a timeout they still wait, bounded, for their own copy to land).
 * ds_set_wait_limits sets both first-wait limits for launches set up
 * afterwards, process-wide; values <= 0 restore the defaults. */
ds_status ds_set_wait_limits(int64_t lookback_polls, int64_t mbarrier_polls);

/* Runs the two kinds of bounded wait on flags nothing ever sets (a look-back
 * predecessor that never publishes; an mbarrier nobody arrives on, with no
 * copy issued), each limited to `polls` (1..2^20): both give up, DS_ERR_TIMEOUT
 * is set in *status, and out[0] = -1 (look-back prefix), out[1] = 0 (barrier
 * not completed).  scratch: >= 272 bytes (cleared here). */
ds_status ds_probe_wait_timeout(int64_t polls, void *scratch, size_t scratch_bytes, int64_t *out,
                                int32_t *status, void *stream);

/* No counterpart in the reference.  *mapped = 1 when `ptr` is page-locked
 * host memory that kernels address at the same value (unified addressing;
 * cudaHostAlloc'd memory, the page-locked memory of the caching allocators),
 * else 0 (device memory, ordinary pageable memory, null).  Such memory may
 * be given as the output arrays of ds_simulate: the spots then go to the host
 * in the kernel's own coalesced stores, with no separate copy.  The kernel
 * only stores to those arrays; they must stay allocated until the stream has
 * passed the call. */
ds_status ds_host_mapped(const void *ptr, int32_t *mapped);

/* Last host-side error message of the calling thread ("" if none). */
const char *ds_last_error(void);
/* Library version string. */
const char *ds_version(void);

#ifdef __cplusplus
}
#endif
#endif /* DIFFSIMS_GB300_H */
