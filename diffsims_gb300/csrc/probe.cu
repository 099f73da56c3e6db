// FP32 FMA throughput probe: the denominator of the FP32 roofline of the
// screening kernel (no counterpart in the reference).  Each thread runs eight
// independent FMA chains; the result is stored so nothing is optimised away.
// Also the query whether a host buffer is addressable by kernels at its own
// address (used to let the orientation kernel write its spots to the host).
#include "common.cuh"

namespace ds {
__global__ void __launch_bounds__(256) fma_probe_kernel(long long iters, float *out) {
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    const float m = 0.999999f, c = 1e-7f;
    for (long long i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
}  // namespace ds

using namespace ds;

extern "C" ds_status ds_probe_fp32_fma(int64_t iters, int32_t blocks, float *out, void *stream) {
    clear_error();
    DS_REQUIRE(out && iters > 0 && blocks > 0, "ds_probe_fp32_fma: bad arguments");
    fma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(iters, out);
    return check_launch("fma_probe_kernel");
}

extern "C" ds_status ds_host_mapped(const void *ptr, int32_t *mapped) {
    clear_error();
    DS_REQUIRE(mapped, "ds_host_mapped: mapped is null");
    *mapped = 0;
    if (!ptr) return DS_OK;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        (void)cudaGetLastError();  // not known to the runtime: not mapped
        return DS_OK;
    }
    *mapped = (a.type == cudaMemoryTypeHost && a.devicePointer == ptr) ? 1 : 0;
    return DS_OK;
}
