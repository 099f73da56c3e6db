// ds_simulate_noalloc: the orientation kernel for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc, or any allocator, on the simulation
// path: a real-time acquisition loop that must not enter the CUDA allocator
// once it runs, or a host application whose own memory manager owns all
// device memory and hands a library only the buffers it asks for up front.
// ds_simulate already allocates nothing itself, but it needs a caller-owned
// scratch buffer; this entry point needs none: its scratch is a fixed static
// device array of DS_NOALLOC_SCRATCH_BYTES defined in this file.  The caller
// still passes the inputs (phase table, quaternions) and the outputs (CSR
// spot arrays).
//
// Costs and limits:
// * every GPU that loads the library holds the array (64 MiB) until the
//   process exits;
// * problems whose scratch does not fit are rejected with
//   DS_ERR_INVALID_ARGUMENT (the per-CTA candidate staging is shrunk first,
//   down to the bitmap fallback, before a call is rejected);
// * all calls share the one array: calls that overlap on the GPU (on
//   different streams, or from different host threads without ordering) race
//   on it.  Calls on one stream are ordered and safe.  Every call clears the
//   parts that must start at zero (look-back tile states, line counters).
// * every call looks the array's device address up with
//   cudaGetSymbolAddress, with the caller's device current (a host-side
//   lookup once the library's device code is loaded on that device), so the
//   address is never stale, also across a cudaDeviceReset.  The first call on
//   a device loads that device code: make it before any stream capture.
#include "common.cuh"

namespace ds {

constexpr size_t DS_NOALLOC_SCRATCH_BYTES = 64ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[DS_NOALLOC_SCRATCH_BYTES];

ds_status simulate_scratch_plan(const ds_sim_params *p, const ds_phase_table *t, long long n_orient,
                                size_t *total, long long *stage_cap, size_t *per_stage);

// Device address of the static scratch on the current device (host code may
// not use the symbol itself as a device pointer).
static ds_status noalloc_scratch(void **out) {
    void *p = nullptr;
    DS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    DS_REQUIRE(p != nullptr, "ds_simulate_noalloc: no device address for the static scratch");
    *out = p;
    return DS_OK;
}

}  // namespace ds

using namespace ds;

extern "C" ds_status ds_simulate_noalloc(const ds_sim_params *p, const ds_phase_table *t, const double *quats,
                                         int64_t n_orient, ds_spots *out, int32_t *status, void *stream) {
    clear_error();
    DS_NVTX_RANGE("ds_simulate_noalloc");
    DS_REQUIRE(p && t && out && status, "ds_simulate_noalloc: null pointer");
    DS_REQUIRE(p->stage_cap >= 0, "ds_simulate_noalloc: stage_cap < 0");
    void *scratch = nullptr;
    ds_status st = noalloc_scratch(&scratch);
    if (st) return st;
    if (n_orient <= 0)  // nothing to plan: ds_simulate only writes the empty CSR (or rejects n_orient < 0)
        return ds_simulate(p, t, quats, n_orient, out, scratch, DS_NOALLOC_SCRATCH_BYTES, status, stream);
    // Fit the scratch into the static array.  Only the per-CTA candidate
    // staging depends on the staging capacity, linearly: take the largest
    // capacity that fits (1 leaves every orientation on the bitmap fallback),
    // then check it with a second plan.
    ds_sim_params q = *p;
    size_t total = 0, per = 0;
    long long cap = 0;
    st = simulate_scratch_plan(&q, t, n_orient, &total, &cap, &per);
    if (st) return st;  // the plan's own status and message
    if (total > DS_NOALLOC_SCRATCH_BYTES) {
        const size_t slack = 512;  // alignment of the two staging arrays
        const size_t fixed = total - per * (size_t)cap;
        if (fixed + per + slack > DS_NOALLOC_SCRATCH_BYTES) {
            set_error("ds_simulate_noalloc: this problem needs at least " + std::to_string(fixed + per) +
                      " bytes of scratch; the static scratch holds " + std::to_string(DS_NOALLOC_SCRATCH_BYTES) +
                      " bytes (use ds_simulate with a caller-owned scratch buffer)");
            return DS_ERR_INVALID_ARGUMENT;
        }
        const long long fit = (long long)((DS_NOALLOC_SCRATCH_BYTES - fixed - slack) / per);
        q.stage_cap = (int32_t)(fit < cap ? fit : cap);
        st = simulate_scratch_plan(&q, t, n_orient, &total, &cap, &per);
        if (st) return st;
        DS_REQUIRE(total <= DS_NOALLOC_SCRATCH_BYTES, "ds_simulate_noalloc: staging plan does not fit the static scratch");
    }
    return ds_simulate(&q, t, quats, n_orient, out, scratch, DS_NOALLOC_SCRATCH_BYTES, status, stream);
}
