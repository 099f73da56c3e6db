// Batched orientation kernel with the precession rotation average compiled in
// (approximate_precession=False): its own instantiations.
#include "simulate_kernel.cuh"

namespace ds {

const void *simulate_batch_kernel_integral(int O, int form) {
    if (form == DS_FORM_FP64) {
        switch (O) {
            case 1: return (const void *)simulate_batch_kernel<1, DS_FORM_FP64, true>;
            case 2: return (const void *)simulate_batch_kernel<2, DS_FORM_FP64, true>;
            case 4: return (const void *)simulate_batch_kernel<4, DS_FORM_FP64, true>;
            default: return (const void *)simulate_batch_kernel<8, DS_FORM_FP64, true>;
        }
    }
    switch (O) {
        case 1: return (const void *)simulate_batch_kernel<1, DS_FORM_MIXED, true>;
        case 2: return (const void *)simulate_batch_kernel<2, DS_FORM_MIXED, true>;
        case 4: return (const void *)simulate_batch_kernel<4, DS_FORM_MIXED, true>;
        case 8: return (const void *)simulate_batch_kernel<8, DS_FORM_MIXED, true>;
        default: return (const void *)simulate_batch_kernel<16, DS_FORM_MIXED, true>;
    }
}

}  // namespace ds
