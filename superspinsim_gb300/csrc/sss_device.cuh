// Device helpers shared by the plain and batched kernels.
#pragma once
#include <cuda_runtime.h>

namespace sss {

// x == 0.0 (either sign) tested on the integer pipe: on this GPU a double
// comparison issues on the FP64 pipe, which the Horner terms saturate.  The
// same result as x == 0.0 for every x (a NaN is not zero).
__device__ __forceinline__ bool is_zero(double x) {
    return (__double_as_longlong(x) << 1) == 0;
}

// Node time of Gauss-Legendre node `node` in fine step r of output sample
// t, in the reference's operation order (generate_simulator.py:158-167,
// 1954-1959): ((t0 + (r*dt)/F) + dt*t) + (dt*node)/F.  Every operation is
// rounded separately (no contraction into FMA) so that the node times -- and
// with them every segment-boundary comparison -- match the host exactly.
__device__ __forceinline__ double node_time(double t0, double dt, int F, int r,
                                            int t, double node) {
    double toff = __ddiv_rn(__dmul_rn((double)r, dt), (double)F);
    double base = __dadd_rn(__dadd_rn(t0, toff), __dmul_rn(dt, (double)t));
    return __dadd_rn(base, __ddiv_rn(__dmul_rn(dt, node), (double)F));
}

// Value of one coefficient channel: segments of (t_end, offset, amplitude,
// frequency, phase); first segment with t < t_end gives
// offset + amplitude*cos(tau*frequency*t + phase), else 0.  The cosine
// argument is rounded step by step as Python's math.tau*f*t + phase is.
__device__ __forceinline__ double segment_value(const double* s, double t) {
    double a = s[2];
    if (is_zero(a)) return s[1];
    double arg = __dadd_rn(__dmul_rn(__dmul_rn(6.283185307179586, s[3]), t), s[4]);
    return __dadd_rn(s[1], __dmul_rn(a, cos(arg)));
}

__device__ __forceinline__ double channel_value(const double* prog, int nseg,
                                                int ch, double t) {
    const double* p = prog + (size_t)ch * nseg * 5;
    for (int s = 0; s < nseg; s++, p += 5)
        if (t < p[0]) return segment_value(p, t);
    return 0.0;
}

}  // namespace sss
