// Slot-programmed adjoint backward kernel: the row-part adjoint's backward
// sweep (sss_adjoint.cu, k_adjoint_parts) with each exponential's block
// series run on a slot program of the block matrix [[Omega^T, G^T],
// [0, Omega^T]] (sss_adjoint_slots.cuh).  Per group of L lanes one
// trajectory, walking its stored forward states backwards:
//   - at every output sample the readout weight joins the adjoint (py rows);
//   - per exponential the block series runs in scaled Horner form from
//     V = [0; mu], leaving [L(Omega^T, G^T) mu; E^T mu] in V;
//   - g = rho_before . px; the px rows return to zero for the next
//     exponential;
//   - per quadrature node the gradient sums of the differentiated channel's
//     current segment grow by h W[e,k] (dc/dtheta) g, every lane keeping its
//     share, summed over the group when the node's segment changes.
// The channel values and derivative factors come from a ring filled kRing
// steps at a time walking back, as in k_adjoint_parts.
#include <cuda_runtime.h>
#include <math.h>

#include "sss_adjoint_ring.cuh"
#include "sss_adjoint_slots.cuh"
#include "sss_slots.cuh"

namespace sss {
namespace {

template <int L, class Prog>
__global__ void __launch_bounds__(256, 1) k_adjoint_slots(const AdjSlotArgs a) {
    extern __shared__ double smem[];
    constexpr int S = Prog::kSlots;
    const int M = a.M, M2 = a.M2, Ms = a.Ms, NL = a.n_live, K = a.K, Q = a.Q, d = a.degree;
    const int slot = threadIdx.x / L, li = threadIdx.x % L;
    const size_t per_slot = (3 * (size_t)Ms + (size_t)kRing * (Q * NL + K * NL + 4 * Q)) | 1;
    double* V = smem + slot * per_slot;
    double* A = V + Ms;
    double* B = A + Ms;
    double* ringc = V + 3 * (size_t)Ms;         // [s][k][live] node values
    double* ring_ag = ringc + kRing * Q * NL;   // [s][e][live] CF weights
    double* ring_d = ring_ag + kRing * K * NL;  // [s][k][4] cos, -a sin, segment, -a sin tau t
    double* s_rw = smem + (size_t)(blockDim.x / L) * per_slot;
    for (int i = threadIdx.x; i < M; i += blockDim.x) s_rw[i] = a.rw[i];
    for (int i = li; i < 3 * Ms; i += L) V[i] = 0.0;
    char* const sb = reinterpret_cast<char*>(smem);
    const int oV = (int)((char*)V - sb), oA = (int)((char*)A - sb), oB = (int)((char*)B - sb);
    const int MsB = Ms * (int)sizeof(double);
    Prog program;
    program.decode(a.cw, L, li, M2, oV, oA, oB);
    // this lane's forward rows and block rows (even splits: every per-row
    // loop sits between group barriers)
    const int f0 = (int)((long)M * li / L), f1 = (int)((long)M * (li + 1) / L);
    const int b0 = (int)((long)M2 * li / L), b1 = (int)((long)M2 * (li + 1) / L);
    constexpr int kPre = 4;
    int fp[kPre], px[kPre], py[kPre];
#pragma unroll
    for (int i = 0; i < kPre; i++) {
        const bool own = f0 + i < f1;
        fp[i] = own ? __ldg(a.fpos + f0 + i) : 0;
        px[i] = own ? __ldg(a.ppx + f0 + i) : 0;
        py[i] = own ? __ldg(a.ppy + f0 + i) : 0;
    }
    __syncthreads();

    constexpr bool kCta = L > 32;
    const unsigned lane_in_warp = threadIdx.x & 31;
    const unsigned leader = kCta ? 0u : lane_in_warp / L * L;
    const unsigned gmask = (L >= 32) ? 0xffffffffu : (((1u << L) - 1u) << leader);
    __shared__ int s_bcast;
    __shared__ double s_red[kCta ? L / 32 : 1];
    auto gsync = [&]() {
        if (kCta) __syncthreads(); else __syncwarp(gmask);
    };
    // sum over the group, valid in lane 0
    auto gsum = [&](double v) {
#pragma unroll
        for (int o = (L < 32 ? L : 32) / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o);
        if (kCta) {
            if (lane_in_warp == 0) s_red[threadIdx.x >> 5] = v;
            __syncthreads();
            if (threadIdx.x == 0)
                for (int w = 1; w < L / 32; w++) v += s_red[w];
            __syncthreads();
        }
        return v;
    };
    auto lds = [&](int off) { return *reinterpret_cast<const double*>(sb + off); };
    auto sts = [&](int off, double x) { *reinterpret_cast<double*>(sb + off) = x; };
    double om[S];

    while (true) {
        int nb = 0;
        if (li == 0) nb = atomicAdd(a.queue, 1);
        if (kCta) {
            if (li == 0) s_bcast = nb;
            __syncthreads();
            nb = s_bcast;
            __syncthreads();
        } else {
            nb = __shfl_sync(gmask, nb, leader);
        }
        const int b = nb;
        if (b >= a.ntraj) break;
        const double* prog = a.prog + (size_t)b * a.nch * a.nseg * 5;
        const double* dprog = prog + (size_t)a.dch * a.nseg * 5;
        // objective from the forward readouts
        {
            double s = 0.0;
            for (int t = li; t < a.T; t += L) s = fma(a.tw[t], a.readout[(size_t)b * a.T + t], s);
            s = gsum(s);
            if (li == 0) a.J[b] = s;
        }
        double* gb = a.grad + (size_t)b * a.nseg * a.npar;
        int cur_seg[kMaxQ];
        double acc_a[kMaxQ], acc_p[kMaxQ], acc_o[kMaxQ], acc_f[kMaxQ];
#pragma unroll
        for (int k = 0; k < kMaxQ; k++) {
            cur_seg[k] = -1;
            acc_a[k] = acc_p[k] = acc_o[k] = acc_f[k] = 0.0;
        }
        auto flush = [&](int k) {
            const double ta = gsum(acc_a[k]), tp = gsum(acc_p[k]);
            double to = 0.0, tf = 0.0;
            if (a.npar == 4) {
                to = gsum(acc_o[k]);
                tf = gsum(acc_f[k]);
            }
            if (li == 0) {
                double* gs = gb + (size_t)a.npar * cur_seg[k];
                gs[0] += ta;
                gs[1] += tp;
                if (a.npar == 4) {
                    gs[2] += to;
                    gs[3] += tf;
                }
            }
            acc_a[k] = acc_p[k] = acc_o[k] = acc_f[k] = 0.0;
        };
        // mu = 0, px = 0
        for (int row = b0; row < b1; row++) V[row] = 0.0;
        gsync();
        const double* st_b = a.states + (size_t)b * a.n_steps * K * M;
        int rp = kRing;
        for (long n = a.n_steps - 1; n >= 0; n--) {
            if ((n + 1) % a.F == 0) {
                const double w = a.tw[(n + 1) / a.F - 1];
#pragma unroll
                for (int i = 0; i < kPre; i++)
                    if (f0 + i < f1) V[py[i]] = fma(w, s_rw[f0 + i], V[py[i]]);
                for (int i = f0 + kPre; i < f1; i++) {
                    const int r = __ldg(a.ppy + i);
                    V[r] = fma(w, s_rw[i], V[r]);
                }
                gsync();
            }
            if (rp == kRing) {
                adjoint_ring_nodes(a, prog, dprog, n, li, L, ringc, ring_d);
                gsync();
                adjoint_ring_weights(a, li, L, ringc, ring_ag);
                gsync();
                rp = 0;
            }
            for (int e_exp = 0; e_exp < K; e_exp++) {
                // the state before this exponential, loaded now, used after
                // the series
                const double* rb = st_b + ((size_t)n * K + e_exp) * M;
                double rbv[kPre];
#pragma unroll
                for (int i = 0; i < kPre; i++) rbv[i] = f0 + i < f1 ? __ldg(rb + fp[i]) : 0.0;
                const double* o0 = a.om0 + (size_t)e_exp * S * L + li;
#pragma unroll
                for (int q = 0; q < S; q++) om[q] = __ldg(o0 + (size_t)q * L);
                for (int gi = 0; gi < NL; gi++) {
                    const double c = ring_ag[(rp * K + e_exp) * NL + gi];
                    if (is_zero(c)) continue;
                    const double* gv = a.gv + (size_t)a.live[gi] * S * L + li;
                    const unsigned am = a.amask[gi];
#pragma unroll
                    for (int q = 0; q < S; q++)
                        if ((am >> q) & 1u) om[q] = fma(c, __ldg(gv + (size_t)q * L), om[q]);
                }
                // the block series on V = [0; mu], scaled Horner form as in
                // the forward kernels: V -> A, then A -> B, B -> A, ...
                program.template term<0>(om, d == 1 ? 0.0 : a.cfac[d], 0, lds, sts, gsync);
                int j = d - 1;
                for (; j >= 2; j -= 2) {
                    program.template term<1>(om, a.cfac[j], MsB, lds, sts, gsync);
                    program.template term<2>(om, j == 2 ? 0.0 : a.cfac[j - 1], 0, lds, sts, gsync);
                }
                if (j == 1) program.template term<1>(om, 0.0, MsB, lds, sts, gsync);
                const double* res = (d & 1) ? A : B;
                for (int row = b0; row < b1; row++) V[row] = fma(res[row], a.inv_dfact, V[row]);
                gsync();
                // this lane's share of g = rho_before . px; px back to zero
                double g = 0.0;
#pragma unroll
                for (int i = 0; i < kPre; i++)
                    if (f0 + i < f1) {
                        g = fma(rbv[i], V[px[i]], g);
                        V[px[i]] = 0.0;
                    }
                for (int i = f0 + kPre; i < f1; i++) {
                    const int r = __ldg(a.ppx + i);
                    g = fma(rb[__ldg(a.fpos + i)], V[r], g);
                    V[r] = 0.0;
                }
#pragma unroll
                for (int k = 0; k < kMaxQ; k++) {
                    if (k >= Q) break;
                    const double* rd = ring_d + (rp * Q + k) * 4;
                    const int sg = (int)rd[2];
                    if (sg != cur_seg[k]) {  // the same in every lane of the group
                        if (cur_seg[k] >= 0) flush(k);
                        cur_seg[k] = sg;
                    }
                    if (sg >= 0) {
                        const double hw = a.h * __ldg(a.W + e_exp * Q + k);
                        acc_a[k] = fma(hw * rd[0], g, acc_a[k]);
                        acc_p[k] = fma(hw * rd[1], g, acc_p[k]);
                        acc_o[k] = fma(hw, g, acc_o[k]);
                        acc_f[k] = fma(hw * rd[3], g, acc_f[k]);
                    }
                }
                gsync();
            }
            rp++;
        }
#pragma unroll
        for (int k = 0; k < kMaxQ; k++)
            if (k < Q && cur_seg[k] >= 0) flush(k);
        gsync();
    }
}

template <class Kern>
int launch_adj(sss_plan* p, Kern kern, const AdjSlotArgs& a, int threads, int slots_per_cta,
               size_t smem, cudaStream_t st) {
    SSS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    SSS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
    if (per_sm < 1) return fail(SSS_EINVAL, "adjoint kernel does not fit on an SM");
    const int want = (a.ntraj + slots_per_cta - 1) / slots_per_cta;
    const int grid = std::max(1, std::min(want, per_sm * p->num_sms));
    kern<<<grid, threads, smem, st>>>(a);
    SSS_CUDA(cudaGetLastError());
    return SSS_OK;
}

}  // namespace

int launch_adjoint_slots(sss_plan* p, int L, bool phased, int shape, int S, const AdjSlotArgs& a,
                         int threads, size_t smem, cudaStream_t st) {
    const int spc = threads / L;
    static_assert(kPhasedShapeCount == 8, "one case per phased shape");
#define SSS_ADJ_PHASED(LL, k)                                                                 \
    case k:                                                                                   \
        return launch_adj(p,                                                                  \
                          k_adjoint_slots<LL, PhasedProgram<kPhasedShapes[k].C1,              \
                                                            kPhasedShapes[k].P1,              \
                                                            kPhasedShapes[k].C2,              \
                                                            kPhasedShapes[k].P2>>,            \
                          a, threads, spc, smem, st);
    if (L == 64 && phased) {
        switch (shape) {
            SSS_ADJ_PHASED(64, 0)
            SSS_ADJ_PHASED(64, 1)
            SSS_ADJ_PHASED(64, 2)
            SSS_ADJ_PHASED(64, 3)
            SSS_ADJ_PHASED(64, 4)
            SSS_ADJ_PHASED(64, 5)
            SSS_ADJ_PHASED(64, 6)
            SSS_ADJ_PHASED(64, 7)
            default: return fail(SSS_EINVAL, "no phased adjoint kernel for this shape");
        }
    }
    if (L == 64 && !phased) {
        // one trajectory per 64-thread CTA: for batches too small to give
        // every SM sub-partition a warp at 32 lanes
        switch (S) {
            case 5: return launch_adj(p, k_adjoint_slots<64, SlotProgram<5>>, a, threads, spc, smem, st);
            case 6: return launch_adj(p, k_adjoint_slots<64, SlotProgram<6>>, a, threads, spc, smem, st);
            case 7: return launch_adj(p, k_adjoint_slots<64, SlotProgram<7>>, a, threads, spc, smem, st);
            case 8: return launch_adj(p, k_adjoint_slots<64, SlotProgram<8>>, a, threads, spc, smem, st);
            default: return fail(SSS_EINVAL, "no 64-lane slot-packed adjoint kernel for " +
                                                 std::to_string(S) + " slots");
        }
    }
    if (L != 32) return fail(SSS_EINVAL, "the slot adjoint runs 32- or 64-lane groups");
    if (phased) {
        switch (shape) {
            SSS_ADJ_PHASED(32, 0)
            SSS_ADJ_PHASED(32, 1)
            SSS_ADJ_PHASED(32, 2)
            SSS_ADJ_PHASED(32, 3)
            SSS_ADJ_PHASED(32, 4)
            SSS_ADJ_PHASED(32, 5)
            SSS_ADJ_PHASED(32, 6)
            SSS_ADJ_PHASED(32, 7)
            default: return fail(SSS_EINVAL, "no phased adjoint kernel for this shape");
        }
    }
#undef SSS_ADJ_PHASED
    switch (S) {
        case 8: return launch_adj(p, k_adjoint_slots<32, SlotProgram<8>>, a, threads, spc, smem, st);
        case 10: return launch_adj(p, k_adjoint_slots<32, SlotProgram<10>>, a, threads, spc, smem, st);
        case 12: return launch_adj(p, k_adjoint_slots<32, SlotProgram<12>>, a, threads, spc, smem, st);
        case 14: return launch_adj(p, k_adjoint_slots<32, SlotProgram<14>>, a, threads, spc, smem, st);
        case 16: return launch_adj(p, k_adjoint_slots<32, SlotProgram<16>>, a, threads, spc, smem, st);
        default: return fail(SSS_EINVAL, "no slot-packed adjoint kernel for " + std::to_string(S) + " slots");
    }
}

}  // namespace sss
