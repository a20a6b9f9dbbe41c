// Slot-programmed batched kernels: the slot-packed variant (6) and the
// phased row-part variant (7), included by sss_slots_warp.cu (groups of 8,
// 16 or 32 lanes), sss_slots_cta.cu (64, 128 or 256) and sss_phased.cu.
//
// Every lane of a group runs the same S FMA slots per Horner term.  The
// Taylor action of an exponential is evaluated in scaled Horner form: with
// degree d and u_d = v,
//     u_{j-1} = c_j v + Omega u_j,   c_j = d!/(j-1)!,   e^Omega v ~ u_0 / d!
// (u_j = (d!/j!) w_j for the usual Horner iterates w_{j-1} = v + Omega w_j/j),
// so the v term of a row is one more FMA entry with the uniform coefficient
// c_j and a row of n entries costs n + 1 slots.  The last term drops the v
// term: e^Omega v ~ v + (Omega u_1)/d!.  The host lays the pieces
// of rows out lane by lane (slots_layout_rows, phased_layout_rows in
// sss_batch.cu); per slot a lane loads its operand (an entry of the current
// iterate, of v, or a parked partial sum) and computes
// s = fma(coefficient, operand, s or its piece's start value); where a
// piece ends it stores s (to a row of the next iterate, or to a partial sum
// that a piece after the barrier starts from or adds).
//
// The slot program is decoded once per launch into shared-memory byte
// offsets for each buffer role, so a term is straight-line code.  v stays
// in buffer V for the whole exponential; the iterates alternate between A
// and B (the first term reads V, writes A).  A buffer holds M rows, the
// zero row M, the sink row M+1 and the partial sums at M+2...  Everything
// around the exponential -- coefficient ring, constant part of Omega, work
// queue, rotating frame, readouts, stored states -- is the row-part
// kernel's.
#pragma once
#include "sss_batch_args.cuh"
#include "sss_device.cuh"

namespace sss {
namespace {

// Shared-memory byte offsets of a slot's operand in the three buffer roles
// of a term: the first term (current = V, next = A), current = A (next =
// B), current = B (next = A).
struct SlotLoads {
    int F, A, B;
};
__device__ __forceinline__ SlotLoads slot_loads(unsigned lw, int oV, int oA, int oB) {
    const int off = (int)(lw & 0x3fffu) * (int)sizeof(double);
    const unsigned src = lw & (3u << 14);
    if (src == kLdV) return {oV + off, oV + off, oV + off};
    if (src == kLdNext) return {oA + off, oB + off, oA + off};
    return {oV + off, oA + off, oB + off};
}

// Slot-packed program: S slots; pieces start and end anywhere (a select per
// slot picks the start value); one barrier at slot S/2 (donor pieces end by
// it, receiver pieces start at it or later).
template <int S>
struct SlotProgram {
    static constexpr int kSlots = S, SA = S / 2;
    int ldF[S], ldA[S], ldB[S], stA[S], b0A[S];
    unsigned vmask = 0u, pmask = 0u, smask = 0u, emask = 0u;

    __device__ __forceinline__ void decode(const unsigned* cw, int L, int li, int M, int oV, int oA,
                                           int oB) {
#pragma unroll
        for (int q = 0; q < S; q++) {
            const unsigned lw = __ldg(cw + (size_t)q * L + li);
            const unsigned sw = __ldg(cw + (size_t)(S + q) * L + li);
            const SlotLoads l = slot_loads(lw, oV, oA, oB);
            ldF[q] = l.F;
            ldA[q] = l.A;
            ldB[q] = l.B;
            if ((lw & (3u << 14)) == kLdV) vmask |= 1u << q;
            if ((lw & (3u << 14)) == kLdNext) pmask |= 1u << q;
            stA[q] = oA + (int)(sw & 0x3fffu) * (int)sizeof(double);
            if ((int)(sw & 0x3fffu) != M + 1) emask |= 1u << q;
            b0A[q] = oA + (int)((sw >> 14) & 0x3fffu) * (int)sizeof(double);
            if (sw & kStStart) smask |= 1u << q;
        }
    }

    // One Horner term.  Role 0: current = V, next = A; 1: current = A, next
    // = B; 2: current = B, next = A.  shift: 0 for next = A, the buffer size
    // in bytes for next = B.
    template <int Role, class Ld, class St, class Sync>
    __device__ __forceinline__ void term(const double (&om)[S], double cj, int shift, Ld lds, St sts,
                                         Sync gsync) const {
        const int(&ld)[S] = Role == 0 ? ldF : (Role == 1 ? ldA : ldB);
        double X[S], B0[S];
#pragma unroll
        for (int q = 0; q < S; q++) X[q] = lds(ld[q]);
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < SA; q++) {
            const double base = ((smask >> q) & 1u) ? 0.0 : s;
            const double cf = ((vmask >> q) & 1u) ? cj : om[q];
            s = fma(cf, X[q], base);
            if ((emask >> q) & 1u) sts(stA[q] + shift, s);
        }
        gsync();
#pragma unroll
        for (int q = SA; q < S; q++) {
            if ((pmask >> q) & 1u) X[q] = lds(ld[q]);
            B0[q] = lds(b0A[q] + shift);
        }
#pragma unroll
        for (int q = SA; q < S; q++) {
            const double base = ((smask >> q) & 1u) ? B0[q] : s;
            const double cf = ((vmask >> q) & 1u) ? cj : om[q];
            s = fma(cf, X[q], base);
            if ((emask >> q) & 1u) sts(stA[q] + shift, s);
        }
        gsync();
    }
};

// Phased row-part program: per lane C1 chains of P1 slots (phase 1, each
// from zero), a barrier, then C2 chains of P2 slots (phase 2, each from a
// parked partial sum or zero).  Chains start and end at fixed slots, so the
// FMA chains carry no select; the C1 (C2) chains are interleaved slot by
// slot.  Slot of item e of chain c: e*C1 + c in phase 1, C1*P1 + e*C2 + c
// in phase 2.
template <int C1, int P1, int C2, int P2>
struct PhasedProgram {
    static constexpr int S1 = C1 * P1, kSlots = S1 + C2 * P2, S = kSlots;
    int ldF[S], ldA[S], ldB[S], st1[C1], st2[C2], b02[C2];
    unsigned vmask = 0u, pmask = 0u, e1 = 0u, e2 = 0u;

    __device__ __forceinline__ void decode(const unsigned* cw, int L, int li, int M, int oV, int oA,
                                           int oB) {
#pragma unroll
        for (int q = 0; q < S; q++) {
            const unsigned lw = __ldg(cw + (size_t)q * L + li);
            const SlotLoads l = slot_loads(lw, oV, oA, oB);
            ldF[q] = l.F;
            ldA[q] = l.A;
            ldB[q] = l.B;
            if ((lw & (3u << 14)) == kLdV) vmask |= 1u << q;
            if ((lw & (3u << 14)) == kLdNext) pmask |= 1u << q;
        }
#pragma unroll
        for (int c = 0; c < C1; c++) {
            const unsigned sw = __ldg(cw + (size_t)(S + (P1 - 1) * C1 + c) * L + li);
            st1[c] = oA + (int)(sw & 0x3fffu) * (int)sizeof(double);
            if ((int)(sw & 0x3fffu) != M + 1) e1 |= 1u << c;
        }
#pragma unroll
        for (int c = 0; c < C2; c++) {
            const unsigned s0 = __ldg(cw + (size_t)(S + S1 + c) * L + li);
            const unsigned sw = __ldg(cw + (size_t)(S + S1 + (P2 - 1) * C2 + c) * L + li);
            b02[c] = oA + (int)((s0 >> 14) & 0x3fffu) * (int)sizeof(double);
            st2[c] = oA + (int)(sw & 0x3fffu) * (int)sizeof(double);
            if ((int)(sw & 0x3fffu) != M + 1) e2 |= 1u << c;
        }
    }

    template <int Role, class Ld, class St, class Sync>
    __device__ __forceinline__ void term(const double (&om)[S], double cj, int shift, Ld lds, St sts,
                                         Sync gsync) const {
        const int(&ld)[S] = Role == 0 ? ldF : (Role == 1 ? ldA : ldB);
        double X[S];
#pragma unroll
        for (int q = 0; q < S; q++) X[q] = lds(ld[q]);
        double s1[C1];
#pragma unroll
        for (int e = 0; e < P1; e++)
#pragma unroll
            for (int c = 0; c < C1; c++) {
                const int q = e * C1 + c;
                const double cf = ((vmask >> q) & 1u) ? cj : om[q];
                s1[c] = e == 0 ? cf * X[q] : fma(cf, X[q], s1[c]);
            }
#pragma unroll
        for (int c = 0; c < C1; c++)
            if ((e1 >> c) & 1u) sts(st1[c] + shift, s1[c]);
        gsync();
        double s2[C2];
#pragma unroll
        for (int c = 0; c < C2; c++) s2[c] = lds(b02[c] + shift);
#pragma unroll
        for (int q = S1; q < S; q++)
            if ((pmask >> q) & 1u) X[q] = lds(ld[q]);
#pragma unroll
        for (int e = 0; e < P2; e++)
#pragma unroll
            for (int c = 0; c < C2; c++) {
                const int q = S1 + e * C2 + c;
                const double cf = ((vmask >> q) & 1u) ? cj : om[q];
                s2[c] = fma(cf, X[q], s2[c]);
            }
#pragma unroll
        for (int c = 0; c < C2; c++)
            if ((e2 >> c) & 1u) sts(st2[c] + shift, s2[c]);
        gsync();
    }
};

template <int L, class Prog>
__global__ void __launch_bounds__(256, 1) k_batch_slots(const BatchArgs a) {
    extern __shared__ double smem[];
    constexpr int S = Prog::kSlots;
    const int M = a.M, NL = a.n_live, NC = a.n_lch, K = a.K, Q = a.Q;
    const int Ms = M + 2 + a.npart;  // rows, zero row, sink row, partial sums
    const int slot = threadIdx.x / L, li = threadIdx.x % L;
    const size_t per_slot = (3 * (size_t)Ms + (size_t)kRing * (Q * NC + K * NL)) | 1;
    double* V = smem + slot * per_slot;
    double* A = V + Ms;
    double* B = A + Ms;
    double* ringc = V + 3 * (size_t)Ms;          // [s][k][live channel] node values
    double* ring_ag = ringc + kRing * Q * NC;    // [s][e][live] CF weights
    double* s_rw = smem + (size_t)(blockDim.x / L) * per_slot;
    for (int i = threadIdx.x; i < M; i += blockDim.x) s_rw[i] = a.rw ? a.rw[i] : 0.0;
    for (int i = li; i < 3 * Ms; i += L) V[i] = 0.0;
    char* const sb = reinterpret_cast<char*>(smem);
    const int oV = (int)((char*)V - sb), oA = (int)((char*)A - sb), oB = (int)((char*)B - sb);
    const int MsB = Ms * (int)sizeof(double);
    Prog program;
    program.decode(a.cw, L, li, M, oV, oA, oB);
    const int r0 = __ldg(a.rbeg + li), r1 = __ldg(a.rbeg + li + 1);
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
    int b = -1, T_b = 0, t = 0, r = 0, rp = kRing;
    const double* prog = nullptr;
    auto store_lab = [&](double* dst) {
        for (int i = li; i < a.N; i += L) {
            double o = 0.0;
            for (int row = 0; row < M; row++)
                o = fma(__ldg(a.Vm + (size_t)i * a.N + __ldg(a.row_orig + row)), V[row], o);
            dst[i] = o;
        }
    };

    while (true) {
        if (r == 0 && t >= T_b) {
            if (b >= 0 && a.fin) {
                if (a.rot)
                    store_lab(a.fin + (size_t)b * a.N);
                else
                    for (int row = r0; row < r1; row++) {
                    a.fin[(size_t)b * a.N + a.row_orig[row]] = V[row];
                    note_nonfinite(a, V[row], b, a.t_end);
                }
            }
            if (b >= 0 && a.readout)
                for (int tt = max(T_b, a.t_begin) + li; tt < a.t_end; tt += L)
                    a.readout[(size_t)b * a.T_max + tt] = 0.0;
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
            b = nb;
            if (b >= a.ntraj) break;
            if (a.order) b = __ldg(a.order + b);
            T_b = min(a.samples ? a.samples[b] : a.T_max, a.t_end);
            t = a.t_begin;
            rp = kRing;
            prog = a.prog ? a.prog + (size_t)b * a.nch * a.nseg * 5 : nullptr;
            const double* r0b = a.rho0 + (size_t)b * a.N;
            if (a.rot) {
                for (int row = r0; row < r1; row++) {
                    const double* vi = a.Vinvm + (size_t)__ldg(a.row_orig + row) * a.N;
                    double o = 0.0;
                    for (int j = 0; j < a.N; j++) o = fma(__ldg(vi + j), r0b[j], o);
                    V[row] = o;
                }
            } else {
                for (int row = r0; row < r1; row++) V[row] = r0b[a.row_orig[row]];
            }
            gsync();
            if (t >= T_b) continue;
        }
        if (rp == kRing) {
            for (int i = li; i < kRing * Q * NC; i += L) {
                const int s = i / (Q * NC), rem = i - s * Q * NC, k = rem / NC, ci = rem - k * NC;
                const int rr = r + s, ts = t + rr / a.F, rs = rr % a.F;
                const int ch = a.lch_chan[ci];
                double val = 0.0;
                if (a.tab) {
                    if (ts < a.T_max)
                        val = __ldg(a.tab + (((size_t)b * a.F + rs) * a.T_max + ts) * (size_t)(Q * a.tab_G) +
                                    (size_t)k * a.tab_G + ch);
                } else if (ch < a.nch) {
                    const double tn = __dadd_rn(__dadd_rn(__dadd_rn(a.t0, __ldg(a.toff + rs)),
                                                          __dmul_rn(a.dt, (double)ts)),
                                                __ldg(a.noff + k));
                    val = channel_value(prog, a.nseg, ch, tn);
                }
                ringc[i] = val;
            }
            gsync();
            for (int i = li; i < kRing * K * NL; i += L) {
                const int s = i / (K * NL), rem = i - s * K * NL, e = rem / NL, gi = rem - e * NL;
                const int kk = a.live_k[gi], ci = a.live_ch[gi];
                double w = 0.0;
                if (kk < 0) {
                    for (int k = 0; k < Q; k++)
                        w = fma(__ldg(a.W + e * Q + k), ringc[(s * Q + k) * NC + ci], w);
                } else {
                    w = __ldg(a.W + e * Q + kk) * ringc[(s * Q + kk) * NC + ci];
                }
                ring_ag[i] = w * a.h_sub;
            }
            gsync();
            rp = 0;
        }
        for (int e_exp = K - 1; e_exp >= 0; e_exp--) {
            if (a.states) {
                double* sp = a.states +
                             (((size_t)b * a.st_steps + (size_t)(t - a.t_begin) * a.F + r) * K + e_exp) * M;
                for (int row = r0; row < r1; row++) sp[row] = V[row];
            }
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
            for (int m = 0; m < a.substeps; m++) {
                // Horner terms j = d .. 1: V -> A, then A -> B, B -> A, ...
                // The last term (j = 1) leaves the v term out and computes
                // Omega u_1 alone; the row becomes v + (Omega u_1)/d!, so the
                // rounded 1/d! scales only that small correction and no
                // bias builds up in the state over many exponentials.
                const int d = a.degree;
                program.template term<0>(om, d == 1 ? 0.0 : a.cfac[d], 0, lds, sts, gsync);
                int j = d - 1;
                for (; j >= 2; j -= 2) {
                    program.template term<1>(om, a.cfac[j], MsB, lds, sts, gsync);
                    program.template term<2>(om, j == 2 ? 0.0 : a.cfac[j - 1], 0, lds, sts, gsync);
                }
                if (j == 1) program.template term<1>(om, 0.0, MsB, lds, sts, gsync);
                // Omega u_1 is in A for odd d, B for even d
                const double* res = (d & 1) ? A : B;
                for (int row = r0; row < r1; row++) V[row] = fma(res[row], a.inv_dfact, V[row]);
                gsync();
            }
        }
        if (a.rot) {
            // e^{L0 h} in the eigenbasis: each kept row from itself and its
            // block partner, through A
            for (int row = r0; row < r1; row++) {
                const double xs = V[row], xp = V[__ldg(a.blk_pos + row)];
                const double cs = __ldg(a.blk_self + row), cp = __ldg(a.blk_part + row);
                A[row] = a.resid ? fma(cp, xp, fma(cs, xs, xs)) : fma(cp, xp, cs * xs);
            }
            gsync();
            for (int row = r0; row < r1; row++) V[row] = A[row];
            gsync();
        }
        rp++;
        if (++r == a.F) {
            r = 0;
            if (a.trace) {
                if (a.rot)
                    store_lab(a.trace + ((size_t)b * a.T_max + t) * a.N);
                else
                    for (int row = r0; row < r1; row++)
                        a.trace[((size_t)b * a.T_max + t) * a.N + a.row_orig[row]] = V[row];
            }
            if (a.readout) {
                double s = 0.0;
                for (int row = r0; row < r1; row++) s = fma(s_rw[row], V[row], s);
                s = gsum(s);
                if (li == 0) {
                    a.readout[(size_t)b * a.T_max + t] = s;
                    note_nonfinite(a, s, b, t);
                }
            }
            t++;
        }
    }
}

// Launch the slot-packed kernel for L lanes and S slots (one of kSlotSizes).
template <int L>
int launch_slots_for(sss_plan* p, int S, const BatchArgs& a, int threads, size_t smem,
                     cudaStream_t st) {
    static_assert(sizeof(kSlotSizes) / sizeof(kSlotSizes[0]) == 9, "one case per slot count");
    switch (S) {
        case 4: return launch(p, k_batch_slots<L, SlotProgram<4>>, a, threads, threads / L, smem, st);
        case 5: return launch(p, k_batch_slots<L, SlotProgram<5>>, a, threads, threads / L, smem, st);
        case 6: return launch(p, k_batch_slots<L, SlotProgram<6>>, a, threads, threads / L, smem, st);
        case 7: return launch(p, k_batch_slots<L, SlotProgram<7>>, a, threads, threads / L, smem, st);
        case 8: return launch(p, k_batch_slots<L, SlotProgram<8>>, a, threads, threads / L, smem, st);
        case 10: return launch(p, k_batch_slots<L, SlotProgram<10>>, a, threads, threads / L, smem, st);
        case 12: return launch(p, k_batch_slots<L, SlotProgram<12>>, a, threads, threads / L, smem, st);
        case 14: return launch(p, k_batch_slots<L, SlotProgram<14>>, a, threads, threads / L, smem, st);
        case 16: return launch(p, k_batch_slots<L, SlotProgram<16>>, a, threads, threads / L, smem, st);
        default: return fail(SSS_EINVAL, "no slot-packed kernel for " + std::to_string(S) + " slots");
    }
}

// Launch the phased row-part kernel for L lanes and kPhasedShapes[shape].
template <int L>
int launch_phased_for(sss_plan* p, int shape, const BatchArgs& a, int threads, size_t smem,
                      cudaStream_t st) {
    static_assert(kPhasedShapeCount == 8, "one case per phased shape");
#define SSS_PHASED(k)                                                                            \
    case k:                                                                                      \
        return launch(p,                                                                         \
                      k_batch_slots<L, PhasedProgram<kPhasedShapes[k].C1, kPhasedShapes[k].P1,  \
                                                     kPhasedShapes[k].C2, kPhasedShapes[k].P2>>, \
                      a, threads, threads / L, smem, st);
    switch (shape) {
        SSS_PHASED(0)
        SSS_PHASED(1)
        SSS_PHASED(2)
        SSS_PHASED(3)
        SSS_PHASED(4)
        SSS_PHASED(5)
        SSS_PHASED(6)
        SSS_PHASED(7)
        default: return fail(SSS_EINVAL, "no phased row-part kernel for shape " + std::to_string(shape));
    }
#undef SSS_PHASED
}

}  // namespace
}  // namespace sss
