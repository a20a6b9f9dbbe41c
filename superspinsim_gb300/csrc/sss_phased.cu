// Phased row-part batched kernels for groups of 8, 16 and 32 lanes.  See
// sss_slots.cuh (PhasedProgram) and phased_layout_rows in sss_batch.cu.
#include "sss_slots.cuh"

namespace sss {

int launch_phased(sss_plan* p, int L, int shape, const BatchArgs& a, int threads, size_t smem,
                  cudaStream_t st) {
    switch (L) {
        case 8: return launch_phased_for<8>(p, shape, a, threads, smem, st);
        case 16: return launch_phased_for<16>(p, shape, a, threads, smem, st);
        case 32: return launch_phased_for<32>(p, shape, a, threads, smem, st);
        default: return fail(SSS_EINVAL, "phased row-part groups have 8, 16 or 32 lanes");
    }
}

}  // namespace sss
