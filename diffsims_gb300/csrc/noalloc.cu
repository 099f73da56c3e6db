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
// * the first call on a device looks up the array's device address with
//   cudaGetSymbolAddress (once per device, with that device current); make
//   that first call before any stream capture.
#include <mutex>

#include "common.cuh"

namespace ds {

constexpr size_t DS_NOALLOC_SCRATCH_BYTES = 64ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[DS_NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static void *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {nullptr};
static std::mutex g_noalloc_mutex;

// Device address of the static scratch on the current device (host code may
// not use the symbol itself as a device pointer).
static ds_status noalloc_scratch(void **out) {
    int dev = 0;
    DS_CUDA_TRY(cudaGetDevice(&dev));
    DS_REQUIRE(dev >= 0 && dev < NOALLOC_MAX_DEVICES, "ds_simulate_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_ptr[dev] == nullptr) {
        void *p = nullptr;
        DS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        DS_REQUIRE(p != nullptr, "ds_simulate_noalloc: no device address for the static scratch");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return DS_OK;
}

}  // namespace ds

using namespace ds;

extern "C" ds_status ds_simulate_noalloc(const ds_sim_params *p, const ds_phase_table *t, const double *quats,
                                         int64_t n_orient, ds_spots *out, int32_t *status, void *stream) {
    clear_error();
    DS_REQUIRE(p && t && out && status, "ds_simulate_noalloc: null pointer");
    DS_REQUIRE(p->stage_cap >= 0, "ds_simulate_noalloc: stage_cap < 0");
    void *scratch = nullptr;
    ds_status st = noalloc_scratch(&scratch);
    if (st) return st;
    // Fit the scratch into the static array: shrink the candidate staging
    // (halving; 1 leaves every orientation on the bitmap fallback) until the
    // plan fits, else reject.
    ds_sim_params q = *p;
    long long cap = q.stage_cap > 0 ? q.stage_cap : 24576;
    size_t need = 0;
    for (;;) {
        q.stage_cap = (int32_t)cap;
        need = ds_simulate_scratch_bytes(&q, t, n_orient);
        if (n_orient > 0 && need == 0) {
            // the plan itself failed (e.g. a table too large for one tile)
            set_error("ds_simulate_noalloc: no launch plan for these sizes");
            return DS_ERR_INVALID_ARGUMENT;
        }
        if (need <= DS_NOALLOC_SCRATCH_BYTES) break;
        if (cap == 1) {
            set_error("ds_simulate_noalloc: this problem needs " + std::to_string(need) +
                      " bytes of scratch; the static scratch holds " + std::to_string(DS_NOALLOC_SCRATCH_BYTES) +
                      " bytes (use ds_simulate with a caller-owned scratch buffer)");
            return DS_ERR_INVALID_ARGUMENT;
        }
        cap = cap > 64 ? cap / 2 : 1;
    }
    return ds_simulate(&q, t, quats, n_orient, out, scratch, DS_NOALLOC_SCRATCH_BYTES, status, stream);
}
