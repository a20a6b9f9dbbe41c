// The coefficient ring of the adjoint backward kernels (k_adjoint_parts in
// sss_adjoint.cu, k_adjoint_slots in sss_adjoint_slots.cu): walking back
// from fine step n, the node values of the live channels for steps n,
// n-1, ..., n-kRing+1 and, for the differentiated channel, the derivative
// factors of its current segment at every node.  Args is either kernel's
// argument struct (the fields used here have the same names in both).
#pragma once
#include "sss_device.cuh"
#include "sss_internal.cuh"

namespace sss {

// segment of a channel's program (prog points at the channel) at time t,
// or -1 past its last segment
__device__ __forceinline__ int channel_segment(const double* prog, int nseg, double t) {
    for (int s = 0; s < nseg; s++)
        if (t < prog[s * 5]) return s;
    return -1;
}

// Node values ringc[(s*Q + k)*NL + gi] of the live channels at node k of
// step n - s, and for the differentiated channel (live index x_live)
// ring_d[(s*Q + k)*4 + {0, 1, 2, 3}] = cos, -a sin, segment, -a sin tau t
// of its segment; lane li of L fills every L-th entry.  The node times and
// cosine arguments are rounded operation by operation as the forward
// kernels round them.
template <class Args>
__device__ __forceinline__ void adjoint_ring_nodes(const Args& a, const double* prog,
                                                   const double* dprog, long n, int li, int L,
                                                   double* ringc, double* ring_d) {
    const int Q = a.Q, NL = a.n_live;
    for (int i = li; i < kRing * Q * NL; i += L) {
        const int s = i / (Q * NL), rem = i - s * Q * NL, k = rem / NL, gi = rem - k * NL;
        const long ns = n - s;
        double val = 0.0, cs = 0.0, dph = 0.0, dfr = 0.0;
        int sg = -1;
        if (ns >= 0) {
            const int ts = (int)(ns / a.F), rs = (int)(ns % a.F);
            const double tn = __dadd_rn(__dadd_rn(__dadd_rn(a.t0, __ldg(a.toff + rs)),
                                                  __dmul_rn(a.dt, (double)ts)),
                                        __ldg(a.noff + k));
            const int g = a.gen_index[a.live[gi]];
            if (gi == a.x_live) {
                sg = channel_segment(dprog, a.nseg, tn);
                if (sg >= 0) {
                    const double* q = dprog + sg * 5;
                    const double arg =
                        __dadd_rn(__dmul_rn(__dmul_rn(6.283185307179586, q[3]), tn), q[4]);
                    cs = cos(arg);
                    dph = -q[2] * sin(arg);
                    dfr = dph * (6.283185307179586 * tn);
                    val = q[2] == 0.0 ? q[1] : __dadd_rn(q[1], __dmul_rn(q[2], cs));
                }
            } else {
                val = (g - 1 < a.nch) ? channel_value(prog, a.nseg, g - 1, tn) : 0.0;
            }
        }
        ringc[i] = val;
        if (gi == a.x_live) {
            double* rd = ring_d + (s * Q + k) * 4;
            rd[0] = cs;
            rd[1] = dph;
            rd[2] = (double)sg;
            rd[3] = dfr;
        }
    }
}

// CF weights ring_ag[(s*K + e)*NL + gi] = h sum_k W[e,k] ringc[s][k][gi].
template <class Args>
__device__ __forceinline__ void adjoint_ring_weights(const Args& a, int li, int L,
                                                     const double* ringc, double* ring_ag) {
    const int Q = a.Q, K = a.K, NL = a.n_live;
    for (int i = li; i < kRing * K * NL; i += L) {
        const int s = i / (K * NL), rem = i - s * K * NL, e = rem / NL, gi = rem - e * NL;
        double w = 0.0;
        for (int k = 0; k < Q; k++) w = fma(__ldg(a.W + e * Q + k), ringc[(s * Q + k) * NL + gi], w);
        ring_ag[i] = w * a.h;
    }
}

}  // namespace sss
