// Slot-packed batched kernels for groups of 64, 128 and 256 lanes (one
// trajectory per CTA).  See sss_slots.cuh.
#include "sss_slots.cuh"

namespace sss {

int launch_slots_cta(sss_plan* p, int L, int S, const BatchArgs& a, int threads, size_t smem,
                     cudaStream_t st) {
    switch (L) {
        case 64: return launch_slots_for<64>(p, S, a, threads, smem, st);
        case 128: return launch_slots_for<128>(p, S, a, threads, smem, st);
        case 256: return launch_slots_for<256>(p, S, a, threads, smem, st);
        default: return fail(SSS_EINVAL, "slot-packed CTA groups have 64, 128 or 256 lanes");
    }
}

}  // namespace sss
