// Slot-packed batched kernels for groups of 8, 16 and 32 lanes (one warp
// holds 4, 2 or 1 trajectories).  See sss_slots.cuh.
#include "sss_slots.cuh"

namespace sss {

int launch_slots_warp(sss_plan* p, int L, int S, const BatchArgs& a, int threads, size_t smem,
                      cudaStream_t st) {
    switch (L) {
        case 8: return launch_slots_for<8>(p, S, a, threads, smem, st);
        case 16: return launch_slots_for<16>(p, S, a, threads, smem, st);
        case 32: return launch_slots_for<32>(p, S, a, threads, smem, st);
        default: return fail(SSS_EINVAL, "slot-packed warp groups have 8, 16 or 32 lanes");
    }
}

}  // namespace sss
