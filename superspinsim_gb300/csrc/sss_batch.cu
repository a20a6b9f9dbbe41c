// Batched sweep path: many trajectories of one model in one persistent
// kernel.  There is no single reference counterpart -- the reference runs
// one trajectory per `simulate` call (superspinsim/generate_simulator.py:
// 1508-2200) and a sweep calls `simspins` in a loop (superspinsim/sugar.py:
// 566-583).  The integrator is the reference's: per fine step of length
// h = dt/F, sample the coefficients at the Q Gauss-Legendre nodes, weight
// them with the commutator-free table W (:278-350), and apply the K
// exponentials, exponential K-1 first (:1259-1294).  What differs is how an
// exponential is applied: instead of forming exp(Omega) as a matrix
// (2R = 70 dense N x N squarings per exponential in the reference, :706-724
// and :882-897), its action on the state is summed directly,
//     v <- sum_{j=0..d} Omega^j v / j!   (m sub-steps of Omega/m),
// with d and m chosen from a norm bound so the truncation stays below the
// unit roundoff 2^-53 per exponential.  Omega = h * sum_g a_g G_g is assembled only on
// the union sparsity pattern of the generators that are active in the
// batch (a generator whose coefficient is zero for every trajectory is
// dropped), restricted to the state entries reachable from the initial
// states' support: entries outside it are exact zeros for all time, so
// skipping them changes no result.
//
// FP64 on GB300 issues about 2 DFMA per clock per SM with a 75-cycle
// latency, so the kernels spend FP64 issue slots only on the sparse products
// and keep the FP64 pipe fed:
//
//  * a group of L lanes owns one trajectory and every lane issues useful
//    FMAs (an FP64 warp instruction costs the same issue time however many
//    of its lanes are active);
//  * the series is evaluated in Horner form, w <- v + (Omega w)/j for
//    j = d..1, so closing a row costs one FMA per piece of the row;
//  * the row-part kernel (k_batch_parts, the default) cuts rows into parts
//    of equal length, so every lane runs the same branch-free chains and the
//    longest dependent chain is a part, not a row; the register and
//    shared-memory variants (whole rows per lane) remain for large patterns;
//  * groups take trajectories from a global atomic counter (the device work
//    queue) until it runs dry, so uneven trajectory lengths balance across
//    SMs; the step loop is flat (finishing a trajectory and starting the
//    next is a short branch inside it) so a warp's groups stay converged.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <functional>
#include <numeric>
#include <random>
#include <vector>

#include "sss_banks.h"
#include "sss_batch_args.cuh"
#include "sss_device.cuh"
#include "sss_internal.cuh"

namespace sss {

// ---------------------------------------------------------------------------
// host: sparse pattern of the lab-frame generators
// ---------------------------------------------------------------------------

int build_sparse(sss_plan* p) {
    // lab plans: G generators; rotating plans: Q*G (node, generator) slots,
    // whose entries below 1e-16 of the slot's largest (the rounding left by
    // the basis change) are dropped
    const int N = p->d.N, G = p->rotating ? p->d.Q * p->d.G : p->d.G;
    SparseGenerators& s = p->sparse;
    std::vector<double> drop(G, 0.0);
    if (p->rotating)
        for (int g = 0; g < G; g++) {
            double mx = 0.0;
            for (size_t i = 0; i < (size_t)N * N; i++)
                mx = std::max(mx, std::fabs(p->gens[(size_t)g * N * N + i]));
            drop[g] = 1e-16 * mx;
        }
    s.N = N;
    s.G = G;
    s.row_ptr.assign(N + 1, 0);
    s.col.clear();
    std::vector<std::vector<double>> vals(G);
    for (int r = 0; r < N; r++) {
        for (int c = 0; c < N; c++) {
            bool nz = false;
            for (int g = 0; g < G; g++)
                if (std::fabs(p->gens[((size_t)g * N + r) * N + c]) > drop[g]) nz = true;
            if (!nz) continue;
            s.col.push_back(c);
            for (int g = 0; g < G; g++) {
                const double v = p->gens[((size_t)g * N + r) * N + c];
                vals[g].push_back(std::fabs(v) > drop[g] ? v : 0.0);
            }
        }
        s.row_ptr[r + 1] = (int)s.col.size();
    }
    s.nnz = (int)s.col.size();
    s.val.clear();
    for (int g = 0; g < G; g++) s.val.insert(s.val.end(), vals[g].begin(), vals[g].end());
    return SSS_OK;
}

namespace {



// Entry word: bits 0-15 column (compressed), bits 16-31 (row + 1) when the
// entry closes its row, else 0.
__device__ __forceinline__ int ent_col(unsigned w) { return (int)(w & 0xffffu); }
__device__ __forceinline__ int ent_end(unsigned w) { return (int)(w >> 16); }

// Coefficients of the current fine step at the Q nodes, lab frame
// [1, ch0, ch1, ...] restricted to the active generators.
__device__ __forceinline__ void sample_coefficients(const BatchArgs& a, const double* prog, int t,
                                                    int r, int li, int L, double* coef) {
    for (int i = li; i < a.Q * a.Ga; i += L) {
        int k = i / a.Ga, g = a.gen_index[i - k * a.Ga];
        double val = 1.0;
        if (g > 0) {
            // ((t0 + (r*dt)/F) + dt*t) + (dt*node)/F, each op rounded
            double tn = __dadd_rn(__dadd_rn(__dadd_rn(a.t0, __ldg(a.toff + r)),
                                            __dmul_rn(a.dt, (double)t)),
                                  __ldg(a.noff + k));
            val = (g - 1 < a.nch) ? channel_value(prog, a.nseg, g - 1, tn) : 0.0;
        }
        coef[i] = val;
    }
}

template <int L>
__global__ void __launch_bounds__(256) k_batch_lanes(const BatchArgs a) {
    extern __shared__ double smem[];
    const int M = a.M, Ga = a.Ga, E = a.E;
    const int slot = threadIdx.x / L, li = threadIdx.x % L;
    // CTA-shared: generator values [g][e][l], entry words [e][l], readout
    // weights; then per slot: Omega [e][l], v, two Horner buffers, coefs
    double* s_gv = smem;
    double* s_rw = s_gv + (size_t)Ga * E * L;
    unsigned* s_ent = reinterpret_cast<unsigned*>(s_rw + M);
    const size_t shared_words = (size_t)Ga * E * L + M + ((size_t)E * L + L + 1) / 2;
    const size_t per_slot = ((size_t)E * L + 3 * M + kMaxQ * kMaxG) | 1;
    double* Om = smem + shared_words + slot * per_slot;
    double* v = Om + (size_t)E * L;
    double* bufA = v + M;
    double* bufB = bufA + M;
    double* coef = bufB + M;
    int* s_cnt = reinterpret_cast<int*>(s_ent + (size_t)E * L);

    for (int i = threadIdx.x; i < Ga * E * L; i += blockDim.x) s_gv[i] = a.gv[i];
    for (int i = threadIdx.x; i < E * L; i += blockDim.x) s_ent[i] = a.ent[i];
    for (int i = threadIdx.x; i < L; i += blockDim.x) s_cnt[i] = a.lane_rows[i];
    for (int i = threadIdx.x; i < M; i += blockDim.x) s_rw[i] = a.rw ? a.rw[i] : 0.0;
    __syncthreads();

    const unsigned lane_in_warp = threadIdx.x & 31;
    const unsigned leader = lane_in_warp / L * L;
    const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << leader);
    const int nE = s_cnt[li];  // entries of this lane
    int b = -1, T_b = 0, t = 0, r = 0;
    const double* prog = nullptr;

    while (true) {
        if (r == 0 && t >= T_b) {
            if (b >= 0 && a.fin)
                for (int e = 0; e < nE; e++) {
                    unsigned w = s_ent[e * L + li];
                    if (ent_end(w)) {
                        int row = ent_end(w) - 1;
                        a.fin[(size_t)b * a.N + a.row_orig[row]] = v[row];
                        note_nonfinite(a, v[row], b, a.t_end);
                    }
                }
            if (b >= 0 && a.readout)
                for (int tt = max(T_b, a.t_begin) + li; tt < a.t_end; tt += L)
                    a.readout[(size_t)b * a.T_max + tt] = 0.0;
            int nb = 0;
            if (li == 0) nb = atomicAdd(a.queue, 1);
            nb = __shfl_sync(gmask, nb, leader);
            b = nb;
            if (b >= a.ntraj) break;
            if (a.order) b = __ldg(a.order + b);
            T_b = min(a.samples ? a.samples[b] : a.T_max, a.t_end);
            t = a.t_begin;
            prog = a.prog + (size_t)b * a.nch * a.nseg * 5;
            for (int e = 0; e < nE; e++) {
                unsigned w = s_ent[e * L + li];
                if (ent_end(w)) {
                    int row = ent_end(w) - 1;
                    v[row] = a.rho0[(size_t)b * a.N + a.row_orig[row]];
                }
            }
            __syncwarp(gmask);
            if (t >= T_b) continue;
        }
        sample_coefficients(a, prog, t, r, li, L, coef);
        __syncwarp(gmask);
        for (int e_exp = a.K - 1; e_exp >= 0; e_exp--) {
            double ag[kMaxG];
            for (int g = 0; g < Ga; g++) {
                double s = 0.0;
                for (int k = 0; k < a.Q; k++) s = fma(__ldg(a.W + e_exp * a.Q + k), coef[k * Ga + g], s);
                ag[g] = s * a.h_sub;
            }
            // assemble Omega on this lane's entries
            for (int e = 0; e < nE; e++) {
                double o = 0.0;
                for (int g = 0; g < Ga; g++) o = fma(ag[g], s_gv[((size_t)g * E + e) * L + li], o);
                Om[e * L + li] = o;
            }
            for (int m = 0; m < a.substeps; m++) {
                // Horner: w <- v + (Omega w)/j for j = d..1, starting at w = v
                const double* cur = v;
                double* nxt = bufA;
                for (int j = a.degree; j >= 1; j--) {
                    const double ij = a.inv_j[j];
                    double s = 0.0;
                    for (int e = 0; e < nE; e++) {
                        unsigned w = s_ent[e * L + li];
                        s = fma(Om[e * L + li], cur[ent_col(w)], s);
                        if (ent_end(w)) {
                            int row = ent_end(w) - 1;
                            nxt[row] = fma(s, ij, v[row]);
                            s = 0.0;
                        }
                    }
                    __syncwarp(gmask);
                    cur = nxt;
                    nxt = (nxt == bufA) ? bufB : bufA;
                }
                // cur holds exp(Omega) v on every row; copy my rows into v
                for (int e = 0; e < nE; e++) {
                    unsigned w = s_ent[e * L + li];
                    if (ent_end(w)) {
                        int row = ent_end(w) - 1;
                        v[row] = cur[row];
                    }
                }
                __syncwarp(gmask);
            }
        }
        if (++r == a.F) {
            r = 0;
            if (a.trace) {
                for (int e = 0; e < nE; e++) {
                    unsigned w = s_ent[e * L + li];
                    if (ent_end(w)) {
                        int row = ent_end(w) - 1;
                        a.trace[((size_t)b * a.T_max + t) * a.N + a.row_orig[row]] = v[row];
                    }
                }
            }
            if (a.readout) {
                double s = 0.0;
                for (int e = 0; e < nE; e++) {
                    unsigned w = s_ent[e * L + li];
                    if (ent_end(w)) {
                        int row = ent_end(w) - 1;
                        s = fma(s_rw[row], v[row], s);
                    }
                }
#pragma unroll
                for (int o = L / 2; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
                if (li == 0) {
                    a.readout[(size_t)b * a.T_max + t] = s;
                    note_nonfinite(a, s, b, t);
                }
            }
            t++;
        }
    }
}

// Two-chain register variant: as k_batch_reg1, but each row's entries
// (padded to an even count) are summed in two interleaved chains whose
// partial sums are parked separately and merged in the closing loop --
// twice the independent FMAs in flight per lane.
template <int L, int EPL>
__global__ void __launch_bounds__(256) k_batch_reg(const BatchArgs a) {
    extern __shared__ double smem[];
    const int M = a.M, Ga = a.Ga;
    const int slot = threadIdx.x / L, li = threadIdx.x % L;
    const size_t per_slot = (5 * (size_t)M + kMaxQ * kMaxG) | 1;
    double* v = smem + slot * per_slot;
    double* bufA = v + M;
    double* bufB = bufA + M;
    double* rs0 = bufB + M;
    double* rs1 = rs0 + M;
    double* coef = rs1 + M;
    double* s_rw = smem + (size_t)(blockDim.x / L) * per_slot;
    for (int i = threadIdx.x; i < M; i += blockDim.x) s_rw[i] = a.rw ? a.rw[i] : 0.0;
    unsigned ent[EPL];
#pragma unroll
    for (int e = 0; e < EPL; e++) ent[e] = __ldg(a.ent + (size_t)e * L + li);
    const int nE = __ldg(a.lane_rows + li);
    const int r0 = __ldg(a.rbeg + li), r1 = __ldg(a.rbeg + li + 1);
    __syncthreads();

    const unsigned lane_in_warp = threadIdx.x & 31;
    const unsigned leader = lane_in_warp / L * L;
    const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << leader);
    int b = -1, T_b = 0, t = 0, r = 0;
    const double* prog = nullptr;
    double om[EPL];

    while (true) {
        if (r == 0 && t >= T_b) {
            if (b >= 0 && a.fin)
                for (int row = r0; row < r1; row++) {
                    a.fin[(size_t)b * a.N + a.row_orig[row]] = v[row];
                    note_nonfinite(a, v[row], b, a.t_end);
                }
            if (b >= 0 && a.readout)
                for (int tt = max(T_b, a.t_begin) + li; tt < a.t_end; tt += L)
                    a.readout[(size_t)b * a.T_max + tt] = 0.0;
            int nb = 0;
            if (li == 0) nb = atomicAdd(a.queue, 1);
            nb = __shfl_sync(gmask, nb, leader);
            b = nb;
            if (b >= a.ntraj) break;
            if (a.order) b = __ldg(a.order + b);
            T_b = min(a.samples ? a.samples[b] : a.T_max, a.t_end);
            t = a.t_begin;
            prog = a.prog + (size_t)b * a.nch * a.nseg * 5;
            for (int row = r0; row < r1; row++) v[row] = a.rho0[(size_t)b * a.N + a.row_orig[row]];
            __syncwarp(gmask);
            if (t >= T_b) continue;
        }
        sample_coefficients(a, prog, t, r, li, L, coef);
        __syncwarp(gmask);
        for (int e_exp = a.K - 1; e_exp >= 0; e_exp--) {
            double ag[kMaxG];
            if (Ga <= L) {
                double mine = 0.0;
                if (li < Ga) {
                    for (int k = 0; k < a.Q; k++)
                        mine = fma(__ldg(a.W + e_exp * a.Q + k), coef[k * Ga + li], mine);
                    mine *= a.h_sub;
                }
                for (int g = 0; g < Ga; g++) ag[g] = __shfl_sync(gmask, mine, leader + g);
            } else {
                for (int g = 0; g < Ga; g++) {
                    double s = 0.0;
                    for (int k = 0; k < a.Q; k++) s = fma(__ldg(a.W + e_exp * a.Q + k), coef[k * Ga + g], s);
                    ag[g] = s * a.h_sub;
                }
            }
#pragma unroll
            for (int e = 0; e < EPL; e++) om[e] = 0.0;
            for (int g = 0; g < Ga; g++) {
                const double c = ag[g];
                if (is_zero(c)) continue;
                const double* gv = a.gv + (size_t)g * EPL * L + li;
#pragma unroll
                for (int e = 0; e < EPL; e++)
                    if (e < nE) om[e] = fma(c, __ldg(gv + (size_t)e * L), om[e]);
            }
            for (int m = 0; m < a.substeps; m++) {
                const double* cur = v;
                double* nxt = bufA;
                for (int j = a.degree; j >= 1; j--) {
                    const double ij = a.inv_j[j];
                    double s0 = 0.0, s1 = 0.0;
#pragma unroll
                    for (int e = 0; e < EPL; e += 2) {
                        if (e >= nE) break;
                        s0 = fma(om[e], cur[ent_col(ent[e])], s0);
                        s1 = fma(om[e + 1], cur[ent_col(ent[e + 1])], s1);
                        if (ent_end(ent[e + 1])) {
                            const int row = ent_end(ent[e + 1]) - 1;
                            rs0[row] = s0;
                            rs1[row] = s1;
                            s0 = 0.0;
                            s1 = 0.0;
                        }
                    }
                    for (int row = r0; row < r1; row++) nxt[row] = fma(rs0[row] + rs1[row], ij, v[row]);
                    __syncwarp(gmask);
                    cur = nxt;
                    nxt = (nxt == bufA) ? bufB : bufA;
                }
                for (int row = r0; row < r1; row++) v[row] = cur[row];
                __syncwarp(gmask);
            }
        }
        if (++r == a.F) {
            r = 0;
            if (a.trace)
                for (int row = r0; row < r1; row++)
                    a.trace[((size_t)b * a.T_max + t) * a.N + a.row_orig[row]] = v[row];
            if (a.readout) {
                double s = 0.0;
                for (int row = r0; row < r1; row++) s = fma(s_rw[row], v[row], s);
#pragma unroll
                for (int o = L / 2; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
                if (li == 0) {
                    a.readout[(size_t)b * a.T_max + t] = s;
                    note_nonfinite(a, s, b, t);
                }
            }
            t++;
        }
    }
}

// Single-chain register variant.  Each row is one FMA chain; where a row
// ends, its sum is parked in shared memory (a store, no FP64 issue slot),
// and the lane closes its own rows with one Horner FMA each in a uniform
// loop after the entries -- instead of a divergent FP64 block after every
// entry position.  The per-exponential generator weights are computed once
// per group (lane g computes weight g) and broadcast by shuffles.
template <int L, int EPL>
__global__ void __launch_bounds__(256) k_batch_reg1(const BatchArgs a) {
    extern __shared__ double smem[];
    const int M = a.M, Ga = a.Ga;
    const int slot = threadIdx.x / L, li = threadIdx.x % L;
    const size_t per_slot = (4 * (size_t)M + kMaxQ * kMaxG) | 1;
    double* v = smem + slot * per_slot;
    double* bufA = v + M;
    double* bufB = bufA + M;
    double* rs = bufB + M;
    double* coef = rs + M;
    double* s_rw = smem + (size_t)(blockDim.x / L) * per_slot;
    for (int i = threadIdx.x; i < M; i += blockDim.x) s_rw[i] = a.rw ? a.rw[i] : 0.0;
    unsigned ent[EPL];
#pragma unroll
    for (int e = 0; e < EPL; e++) ent[e] = __ldg(a.ent + (size_t)e * L + li);
    const int nE = __ldg(a.lane_rows + li);
    const int r0 = __ldg(a.rbeg + li), r1 = __ldg(a.rbeg + li + 1);
    __syncthreads();

    const unsigned lane_in_warp = threadIdx.x & 31;
    const unsigned leader = lane_in_warp / L * L;
    const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << leader);
    int b = -1, T_b = 0, t = 0, r = 0;
    const double* prog = nullptr;
    double om[EPL];

    while (true) {
        if (r == 0 && t >= T_b) {
            if (b >= 0 && a.fin)
                for (int row = r0; row < r1; row++) {
                    a.fin[(size_t)b * a.N + a.row_orig[row]] = v[row];
                    note_nonfinite(a, v[row], b, a.t_end);
                }
            if (b >= 0 && a.readout)
                for (int tt = max(T_b, a.t_begin) + li; tt < a.t_end; tt += L)
                    a.readout[(size_t)b * a.T_max + tt] = 0.0;
            int nb = 0;
            if (li == 0) nb = atomicAdd(a.queue, 1);
            nb = __shfl_sync(gmask, nb, leader);
            b = nb;
            if (b >= a.ntraj) break;
            if (a.order) b = __ldg(a.order + b);
            T_b = min(a.samples ? a.samples[b] : a.T_max, a.t_end);
            t = a.t_begin;
            prog = a.prog + (size_t)b * a.nch * a.nseg * 5;
            for (int row = r0; row < r1; row++) v[row] = a.rho0[(size_t)b * a.N + a.row_orig[row]];
            __syncwarp(gmask);
            if (t >= T_b) continue;
        }
        sample_coefficients(a, prog, t, r, li, L, coef);
        __syncwarp(gmask);
        for (int e_exp = a.K - 1; e_exp >= 0; e_exp--) {
            double ag[kMaxG];
            if (Ga <= L) {
                double mine = 0.0;
                if (li < Ga) {
                    for (int k = 0; k < a.Q; k++)
                        mine = fma(__ldg(a.W + e_exp * a.Q + k), coef[k * Ga + li], mine);
                    mine *= a.h_sub;
                }
                for (int g = 0; g < Ga; g++) ag[g] = __shfl_sync(gmask, mine, leader + g);
            } else {
                for (int g = 0; g < Ga; g++) {
                    double s = 0.0;
                    for (int k = 0; k < a.Q; k++) s = fma(__ldg(a.W + e_exp * a.Q + k), coef[k * Ga + g], s);
                    ag[g] = s * a.h_sub;
                }
            }
#pragma unroll
            for (int e = 0; e < EPL; e++) om[e] = 0.0;
            for (int g = 0; g < Ga; g++) {
                const double c = ag[g];
                if (is_zero(c)) continue;
                const double* gv = a.gv + (size_t)g * EPL * L + li;
#pragma unroll
                for (int e = 0; e < EPL; e++)
                    if (e < nE) om[e] = fma(c, __ldg(gv + (size_t)e * L), om[e]);
            }
            for (int m = 0; m < a.substeps; m++) {
                const double* cur = v;
                double* nxt = bufA;
                for (int j = a.degree; j >= 1; j--) {
                    const double ij = a.inv_j[j];
                    double s0 = 0.0;
#pragma unroll
                    for (int e = 0; e < EPL; e++) {
                        if (e >= nE) break;
                        s0 = fma(om[e], cur[ent_col(ent[e])], s0);
                        if (ent_end(ent[e])) {
                            rs[ent_end(ent[e]) - 1] = s0;
                            s0 = 0.0;
                        }
                    }
                    for (int row = r0; row < r1; row++) nxt[row] = fma(rs[row], ij, v[row]);
                    __syncwarp(gmask);
                    cur = nxt;
                    nxt = (nxt == bufA) ? bufB : bufA;
                }
                for (int row = r0; row < r1; row++) v[row] = cur[row];
                __syncwarp(gmask);
            }
        }
        if (++r == a.F) {
            r = 0;
            if (a.trace)
                for (int row = r0; row < r1; row++)
                    a.trace[((size_t)b * a.T_max + t) * a.N + a.row_orig[row]] = v[row];
            if (a.readout) {
                double s = 0.0;
                for (int row = r0; row < r1; row++) s = fma(s_rw[row], v[row], s);
#pragma unroll
                for (int o = L / 2; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
                if (li == 0) {
                    a.readout[(size_t)b * a.T_max + t] = s;
                    note_nonfinite(a, s, b, t);
                }
            }
            t++;
        }
    }
}

// Row-part variant.  Every row of the pruned pattern is cut into parts of
// at most P entries, and lane l of a group holds C parts: C independent FMA
// chains of exactly P entries (short parts are padded with zero entries that
// read the zero row M), issued interleaved, with no branch between entries.
// Each row has one owner lane, which closes it after the parts are parked in
// shared memory: next[row] = v[row] + (1/j)*sum(parts), one FMA per part,
// through kc uniform close slots (a close word is row | part << 16 |
// first << 31; padding slots write the sink row M+1).  The longest dependent
// chain per Horner term is P + kc FMAs instead of the longest row, and every
// lane runs the same straight-line code.  The state lives in three rotating
// buffers per trajectory, so an exponential ends without a copy.
//
// Omega = om0[e] + sum over live generators of a_g G_g: om0 (host table)
// holds L0 (coefficient 1 in the lab frame) and every channel that is
// constant over the batch.  The live coefficients are sampled for kRing fine
// steps at a time, spread over the group's lanes (node values, then the CF
// weights a_g = h sum_k W[e,k] c_k,g), into a per-trajectory ring in shared
// memory, so a step pays the cosine of its drive only once per kRing steps.
template <int L, int C, int P>
__global__ void __launch_bounds__(256, 1) k_batch_parts(const BatchArgs a) {
    extern __shared__ double smem[];
    constexpr int CP = C * P;
    const int M = a.M, NL = a.n_live, NC = a.n_lch, K = a.K, Q = a.Q;
    const int Ms = M + 2;  // rows, the zero row M, the sink row M+1
    const int slot = threadIdx.x / L, li = threadIdx.x % L;
    const size_t per_slot = (3 * (size_t)Ms + L * C + 1 + (size_t)kRing * (Q * NC + K * NL)) | 1;
    double* sbuf = smem + slot * per_slot;
    double* parts = sbuf + 3 * (size_t)Ms;
    double* ringc = parts + L * C + 1;           // [s][k][live channel] node values
    double* ring_ag = ringc + kRing * Q * NC;    // [s][e][live] CF weights
    double* s_rw = smem + (size_t)(blockDim.x / L) * per_slot;
    for (int i = threadIdx.x; i < M; i += blockDim.x) s_rw[i] = a.rw ? a.rw[i] : 0.0;
    for (int i = li; i < 3 * Ms; i += L) sbuf[i] = 0.0;
    for (int i = li; i < L * C + 1; i += L) parts[i] = 0.0;
    int col[CP];
#pragma unroll
    for (int e = 0; e < CP; e++) col[e] = __ldg(a.pcol + (size_t)e * L + li);
    unsigned cw[kCloseMax];
#pragma unroll
    for (int k = 0; k < kCloseMax; k++) cw[k] = __ldg(a.cw + (size_t)k * L + li);
    const int kc = a.kc;
    const int r0 = __ldg(a.rbeg + li), r1 = __ldg(a.rbeg + li + 1);
    __syncthreads();

    // a group of L <= 32 lanes lives in one warp (warp barriers and
    // shuffles); a wider group is the whole CTA (CTA barriers, shared memory)
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
    double* v = sbuf;
    double* x = sbuf + Ms;
    double* y = x + Ms;
    int b = -1, T_b = 0, t = 0, r = 0, rp = kRing;
    const double* prog = nullptr;
    double om[CP];
    // rotating frame: the lab-basis state V x, all N entries spread over the lanes
    auto store_lab = [&](double* dst) {
        for (int i = li; i < a.N; i += L) {
            double o = 0.0;
            for (int row = 0; row < M; row++)
                o = fma(__ldg(a.Vm + (size_t)i * a.N + __ldg(a.row_orig + row)), v[row], o);
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
                    a.fin[(size_t)b * a.N + a.row_orig[row]] = v[row];
                    note_nonfinite(a, v[row], b, a.t_end);
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
                // eigenbasis coordinates x = V^-1 rho0 on the kept rows
                for (int row = r0; row < r1; row++) {
                    const double* vi = a.Vinvm + (size_t)__ldg(a.row_orig + row) * a.N;
                    double o = 0.0;
                    for (int j = 0; j < a.N; j++) o = fma(__ldg(vi + j), r0b[j], o);
                    v[row] = o;
                }
            } else {
                for (int row = r0; row < r1; row++) v[row] = r0b[a.row_orig[row]];
            }
            gsync();
            if (t >= T_b) continue;
        }
        if (rp == kRing) {
            // node values of the live channels for fine steps (t, r) .. +kRing-1:
            // the program at node time ((t0 + (r*dt)/F) + dt*t) + (dt*node)/F,
            // each op rounded, or the table's row (steps past the last sample
            // of the table read as zero; a trajectory never uses them)
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
            // CF weights: lab generators sum their channel over the nodes; a
            // rotating slot belongs to one node k and takes W[e,k] c_k
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
                for (int row = r0; row < r1; row++) sp[row] = v[row];
            }
            const double* o0 = a.om0 + (size_t)e_exp * CP * L + li;
#pragma unroll
            for (int e = 0; e < CP; e++) om[e] = __ldg(o0 + (size_t)e * L);
            for (int gi = 0; gi < NL; gi++) {
                const double c = ring_ag[(rp * K + e_exp) * NL + gi];
                if (is_zero(c)) continue;
                const double* gv = a.gv + (size_t)a.live[gi] * CP * L + li;
#pragma unroll
                for (int e = 0; e < CP; e++) om[e] = fma(c, __ldg(gv + (size_t)e * L), om[e]);
            }
            for (int m = 0; m < a.substeps; m++) {
                double* cur = v;
                double* nxt = x;
                for (int j = a.degree; j >= 1; j--) {
                    const double ij = a.inv_j[j];
                    double s[C];
#pragma unroll
                    for (int c = 0; c < C; c++) s[c] = 0.0;
#pragma unroll
                    for (int q = 0; q < P; q++)
#pragma unroll
                        for (int c = 0; c < C; c++) s[c] = fma(om[c * P + q], cur[col[c * P + q]], s[c]);
#pragma unroll
                    for (int c = 0; c < C; c++) parts[li * C + c] = s[c];
                    gsync();
                    double acc = 0.0;
#pragma unroll
                    for (int k = 0; k < kCloseMax; k++) {
                        if (k >= kc) break;
                        const unsigned w = cw[k];
                        const int row = (int)(w & 0xffffu);
                        const double base = (w >> 31) ? v[row] : acc;
                        acc = fma(parts[(w >> 16) & 0x7fffu], ij, base);
                        nxt[row] = acc;
                    }
                    gsync();
                    cur = nxt;
                    nxt = (nxt == x) ? y : x;
                }
                // cur holds the new state: it becomes v, the old v a scratch buffer
                if (cur == x) x = v; else y = v;
                v = cur;
            }
        }
        if (a.rot) {
            // e^{L0 h} in the eigenbasis (generate_simulator.py:901-964): 2 x 2
            // blocks of the complex pairs and the real singles, each row from
            // itself and its partner; residual form x + (c_s x + c_p x_p)
            for (int row = r0; row < r1; row++) {
                const double xs = v[row], xp = v[__ldg(a.blk_pos + row)];
                const double cs = __ldg(a.blk_self + row), cp = __ldg(a.blk_part + row);
                x[row] = a.resid ? fma(cp, xp, fma(cs, xs, xs)) : fma(cp, xp, cs * xs);
            }
            gsync();
            double* tmp = v;
            v = x;
            x = tmp;
        }
        rp++;
        if (++r == a.F) {
            r = 0;
            if (a.trace) {
                if (a.rot)
                    store_lab(a.trace + ((size_t)b * a.T_max + t) * a.N);
                else
                    for (int row = r0; row < r1; row++)
                        a.trace[((size_t)b * a.T_max + t) * a.N + a.row_orig[row]] = v[row];
            }
            if (a.readout) {
                double s = 0.0;
                for (int row = r0; row < r1; row++) s = fma(s_rw[row], v[row], s);
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

// Register-state form of the row-part kernel, for one trajectory per warp
// (32 lanes, one chain of P entries per lane) when no lane owns more than
// one row (NV-7: 19 rows in 29 parts).  Each row's value lives in a
// register of its owner lane and moves by warp shuffles: a part fetches its
// columns from their owners, and an owner fetches its row's partial sums
// from the part lanes (padding close slots fetch from a lane whose parts are
// all padding, so they add zero).  There is no shared-memory state, no
// barrier inside a Horner term and no bank conflict; the coefficient ring
// is the row-part kernel's.  Lab frame, no stored states.
template <int P>
__global__ void __launch_bounds__(256, 1) k_batch_shfl(const BatchArgs a) {
    extern __shared__ double smem[];
    constexpr int L = 32;
    constexpr unsigned kFull = 0xffffffffu;
    const int M = a.M, NL = a.n_live, NC = a.n_lch, K = a.K, Q = a.Q;
    const int Ms = M + 2;
    const int slot = threadIdx.x / L, li = threadIdx.x % L;
    // the row-part kernel's per-trajectory layout (only the ring is used)
    const size_t per_slot = (3 * (size_t)Ms + L + 1 + (size_t)kRing * (Q * NC + K * NL)) | 1;
    double* ringc = smem + slot * per_slot + 3 * (size_t)Ms + L + 1;
    double* ring_ag = ringc + kRing * Q * NC;
    double* s_rw = smem + (size_t)(blockDim.x / L) * per_slot;
    for (int i = threadIdx.x; i < M; i += blockDim.x) s_rw[i] = a.rw ? a.rw[i] : 0.0;
    const int r0 = __ldg(a.rbeg + li), r1 = __ldg(a.rbeg + li + 1);
    const int my_row = r1 > r0 ? r0 : -1;
    // owner lane of each part column (the zero row: this lane, weight 0)
    int src[P];
    bool all_pad = true;
#pragma unroll
    for (int q = 0; q < P; q++) {
        const int c = __ldg(a.pcol + (size_t)q * L + li);
        int owner = li;
        if (c < M) {
            all_pad = false;
            for (int l = 0; l < L; l++)
                if (__ldg(a.rbeg + l) <= c && c < __ldg(a.rbeg + l + 1)) owner = l;
        }
        src[q] = owner;
    }
    const unsigned pad_lanes = __ballot_sync(kFull, all_pad);
    const int zero_lane = pad_lanes ? __ffs(pad_lanes) - 1 : li;
    int pl[kCloseMax];
#pragma unroll
    for (int k = 0; k < kCloseMax; k++) {
        const int part = (int)((__ldg(a.cw + (size_t)k * L + li) >> 16) & 0x7fffu);
        pl[k] = part < L ? part : zero_lane;
    }
    const int kc = a.kc;
    __syncthreads();

    int b = -1, T_b = 0, t = 0, r = 0, rp = kRing;
    const double* prog = nullptr;
    double om[P];
    double v = 0.0;  // this lane's row of the state
    while (true) {
        if (r == 0 && t >= T_b) {
            if (b >= 0 && a.fin && my_row >= 0) {
                a.fin[(size_t)b * a.N + a.row_orig[my_row]] = v;
                note_nonfinite(a, v, b, a.t_end);
            }
            if (b >= 0 && a.readout)
                for (int tt = max(T_b, a.t_begin) + li; tt < a.t_end; tt += L)
                    a.readout[(size_t)b * a.T_max + tt] = 0.0;
            int nb = 0;
            if (li == 0) nb = atomicAdd(a.queue, 1);
            nb = __shfl_sync(kFull, nb, 0);
            b = nb;
            if (b >= a.ntraj) break;
            if (a.order) b = __ldg(a.order + b);
            T_b = min(a.samples ? a.samples[b] : a.T_max, a.t_end);
            t = a.t_begin;
            rp = kRing;
            prog = a.prog ? a.prog + (size_t)b * a.nch * a.nseg * 5 : nullptr;
            v = my_row >= 0 ? a.rho0[(size_t)b * a.N + a.row_orig[my_row]] : 0.0;
            __syncwarp(kFull);
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
            __syncwarp(kFull);
            for (int i = li; i < kRing * K * NL; i += L) {
                const int s = i / (K * NL), rem = i - s * K * NL, e = rem / NL, gi = rem - e * NL;
                const int ci = a.live_ch[gi];
                double w = 0.0;
                for (int k = 0; k < Q; k++) w = fma(__ldg(a.W + e * Q + k), ringc[(s * Q + k) * NC + ci], w);
                ring_ag[i] = w * a.h_sub;
            }
            __syncwarp(kFull);
            rp = 0;
        }
        for (int e_exp = K - 1; e_exp >= 0; e_exp--) {
            const double* o0 = a.om0 + (size_t)e_exp * P * L + li;
#pragma unroll
            for (int e = 0; e < P; e++) om[e] = __ldg(o0 + (size_t)e * L);
            for (int gi = 0; gi < NL; gi++) {
                const double c = ring_ag[(rp * K + e_exp) * NL + gi];
                if (is_zero(c)) continue;
                const double* gv = a.gv + (size_t)a.live[gi] * P * L + li;
#pragma unroll
                for (int e = 0; e < P; e++) om[e] = fma(c, __ldg(gv + (size_t)e * L), om[e]);
            }
            for (int m = 0; m < a.substeps; m++) {
                // Horner: w <- v + (Omega w)/j for j = d..1, starting at w = v
                double cur = v;
                for (int j = a.degree; j >= 1; j--) {
                    const double ij = a.inv_j[j];
                    double s = 0.0;
#pragma unroll
                    for (int q = 0; q < P; q++) s = fma(om[q], __shfl_sync(kFull, cur, src[q]), s);
                    double acc = v;
#pragma unroll
                    for (int k = 0; k < kCloseMax; k++) {
                        if (k >= kc) break;
                        acc = fma(__shfl_sync(kFull, s, pl[k]), ij, acc);
                    }
                    cur = acc;
                }
                v = cur;
            }
        }
        rp++;
        if (++r == a.F) {
            r = 0;
            if (a.trace && my_row >= 0)
                a.trace[((size_t)b * a.T_max + t) * a.N + a.row_orig[my_row]] = v;
            if (a.readout) {
                double s = my_row >= 0 ? s_rw[my_row] * v : 0.0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
                if (li == 0) {
                    a.readout[(size_t)b * a.T_max + t] = s;
                    note_nonfinite(a, s, b, t);
                }
            }
            t++;
        }
    }
}



template <int L>
int launch_parts(sss_plan* p, int C, int P, const BatchArgs& a, int threads, size_t smem,
                 cudaStream_t st) {
    static_assert(sizeof(kPartShapes) / sizeof(kPartShapes[0]) == 4, "one case per part shape");
    if (C == 1 && P == 4) return launch(p, k_batch_parts<L, 1, 4>, a, threads, threads / L, smem, st);
    if (C == 2 && P == 4) return launch(p, k_batch_parts<L, 2, 4>, a, threads, threads / L, smem, st);
    if (C == 4 && P == 4) return launch(p, k_batch_parts<L, 4, 4>, a, threads, threads / L, smem, st);
    if (C == 2 && P == 8) return launch(p, k_batch_parts<L, 2, 8>, a, threads, threads / L, smem, st);
    return fail(SSS_EINVAL, "no row-part kernel for this shape");
}

template <int L>
int launch_reg(sss_plan* p, int epl, const BatchArgs& a, int threads, size_t smem, cudaStream_t st,
               bool one_chain) {
    if (one_chain) {
        switch (epl) {
            case 8: return launch(p, k_batch_reg1<L, 8>, a, threads, threads / L, smem, st);
            case 16: return launch(p, k_batch_reg1<L, 16>, a, threads, threads / L, smem, st);
            case 32: return launch(p, k_batch_reg1<L, 32>, a, threads, threads / L, smem, st);
            default: return launch(p, k_batch_reg1<L, 64>, a, threads, threads / L, smem, st);
        }
    }
    switch (epl) {
        case 8: return launch(p, k_batch_reg<L, 8>, a, threads, threads / L, smem, st);
        case 16: return launch(p, k_batch_reg<L, 16>, a, threads, threads / L, smem, st);
        case 32: return launch(p, k_batch_reg<L, 32>, a, threads, threads / L, smem, st);
        default: return launch(p, k_batch_reg<L, 64>, a, threads, threads / L, smem, st);
    }
}

}  // namespace

// Truncation tolerance of the Taylor series per exponential: the unit
// roundoff 2^-53, the tolerance of the truncated-Taylor action of the
// matrix exponential (Al-Mohy & Higham, SIAM J. Sci. Comput. 33(2), 2011).
// The series error then stays below the rounding of a single step.
constexpr double kTaylorTol = 0x1p-53;

// Taylor degree and sub-steps for a norm bound `beta` of Omega: the
// smallest d*m with m*(beta/m)^(d+1)/(d+1)! <= kTaylorTol.
static void choose_taylor(double beta, int forced_degree, int* degree, int* substeps) {
    if (forced_degree > 0) {
        *degree = std::min(forced_degree, kMaxTaylor);
        int m = 1;
        while (m < 1024) {
            double x = beta / m, term = 1.0;
            for (int j = 1; j <= *degree + 1; j++) term *= x / j;
            if (m * term <= kTaylorTol) break;
            m++;
        }
        *substeps = m;
        return;
    }
    int best_d = kMaxTaylor, best_m = 1024;
    for (int m = 1; m <= 1024; m++) {
        double x = beta / m, term = 1.0;
        for (int d = 1; d <= kMaxTaylor; d++) {
            term *= x / d;
            double next = term * x / (d + 1);
            if (m * next <= kTaylorTol) {
                if (d * m < best_d * best_m) { best_d = d; best_m = m; }
                break;
            }
        }
        if (best_d * best_m <= m) break;
    }
    *degree = best_d;
    *substeps = best_m;
}

// Row-part layout of a row pattern `rows` (per reachable row: compressed
// column and SparseGenerators index of each entry): rows cut into parts of
// at most P entries, parts spread over the L*C lane slots (part j -> lane
// j % L, chain j / L), rows given to owner lanes by longest-processing-time
// first on their close cost (one slot per part, one for an empty row).
// Picks the (C, P) shape minimising w_chain*C*P + w_close*kc (FP64
// instructions per Horner term), then the shortest chain P + kc.  Entries
// flagged in `prio` (may be empty) are spread evenly over their row's parts
// and placed first in each part; `nprio` returns the most flagged entries
// in any part.  Fills newpos/row_orig (owner order), lane_of, pcol, cw, gv
// (for `active`), entry_q, C, P, kc, L, E = C*P, threads.
int parts_layout_rows(sss_plan* p, const std::vector<std::vector<BatchLayout::Ent>>& rows,
                      const std::vector<std::vector<char>>& prio, int L, int threads, int w_chain,
                      int w_close, const std::vector<int>& active,
                      const std::vector<int>& rows_reached, BatchLayout* out, int* nprio) {
    BatchLayout& Ly = *out;
    const SparseGenerators& sp = p->sparse;
    const int M = (int)rows.size(), Ga = (int)active.size();
    if (L != 8 && L != 16 && L != 32 && L != 64 && L != 128 && L != 256)
        return fail(SSS_EINVAL, "row-part variant needs 8 to 256 lanes per trajectory (a power of two)");
    if (L > 32) threads = L;  // a group wider than a warp is one CTA
    if (threads % L) return fail(SSS_EINVAL, "CTA size must be a multiple of the lanes per trajectory");
    auto nparts = [&](int i, int P) { return ((int)rows[i].size() + P - 1) / P; };
    // owners by LPT on close cost; returns kc
    auto owners = [&](int P, std::vector<std::vector<int>>* own) {
        std::vector<int> order(M);
        std::iota(order.begin(), order.end(), 0);
        auto cost = [&](int i) { return std::max(1, nparts(i, P)); };
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
        std::vector<int> load(L, 0);
        own->assign(L, {});
        for (int i : order) {
            int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            load[l] += cost(i);
            (*own)[l].push_back(i);
        }
        for (auto& o : *own) std::sort(o.begin(), o.end());
        return M ? *std::max_element(load.begin(), load.end()) : 0;
    };
    int bC = 0, bP = 0, bkc = 0;
    long best_cost = -1, best_path = 0;
    for (const auto& sh : kPartShapes) {
        const int C = sh[0], P = sh[1];
        long total = 0;
        for (int i = 0; i < M; i++) total += nparts(i, P);
        if (total > (long)L * C) continue;
        std::vector<std::vector<int>> own;
        const int kc = owners(P, &own);
        if (kc > kCloseMax) continue;
        const long cost = (long)w_chain * C * P + (long)w_close * kc, path = P + kc;
        if (best_cost < 0 || cost < best_cost || (cost == best_cost && path < best_path)) {
            best_cost = cost; best_path = path; bC = C; bP = P; bkc = kc;
        }
    }
    if (best_cost < 0)
        return fail(SSS_EINVAL, "row-part variant does not fit this pattern at " + std::to_string(L) +
                                    " lanes per trajectory");
    const int C = bC, P = bP, CP = C * P;
    std::vector<std::vector<int>> own;
    owners(P, &own);
    // rows renumbered in owner order: lane l owns [rbeg[l], rbeg[l+1])
    std::vector<int>& newpos = Ly.newpos;
    std::vector<int>& row_orig = Ly.row_orig;
    newpos.assign(M, 0);
    row_orig.assign(M, 0);
    {
        int k = 0;
        for (int l = 0; l < L; l++)
            for (int i : own[l]) { newpos[i] = k; row_orig[k] = rows_reached[i]; k++; }
    }
    Ly.pcol.assign((size_t)CP * L, M);
    Ly.entry_q.assign((size_t)CP * L, -1);
    Ly.gv.assign((size_t)Ga * CP * L, 0.0);
    std::vector<std::vector<int>> part_slots(M);  // per row: smem slot lane*C + c of each part
    int most = 0;
    {
        int j = 0;
        for (int i = 0; i < M; i++) {
            const auto& ents = rows[i];
            const int n = (int)ents.size(), np = nparts(i, P);
            if (np == 0) continue;
            // entries of each part: flagged entries dealt round-robin first,
            // then the others fill up to the part sizes
            std::vector<int> size(np), order_f, order_o;
            for (int q = 0; q < np; q++) size[q] = n / np + (q < n % np ? 1 : 0);
            for (int e = 0; e < n; e++)
                (!prio.empty() && prio[i][e] ? order_f : order_o).push_back(e);
            std::vector<std::vector<int>> pe(np);
            int q = 0;
            for (int e : order_f) {
                for (int tries = 0; (int)pe[q].size() >= size[q] && tries < np; tries++) q = (q + 1) % np;
                pe[q].push_back(e);
                q = (q + 1) % np;
            }
            for (int qq = 0; qq < np; qq++) most = std::max(most, (int)pe[qq].size());
            size_t oi = 0;
            for (int qq = 0; qq < np; qq++)
                while ((int)pe[qq].size() < size[qq]) pe[qq].push_back(order_o[oi++]);
            for (int qq = 0; qq < np; qq++) {
                const int lane = j % L, c = j / L;
                for (int e = 0; e < (int)pe[qq].size(); e++) {
                    const BatchLayout::Ent& en = ents[pe[qq][e]];
                    const size_t idx = (size_t)(c * P + e) * L + lane;
                    Ly.pcol[idx] = newpos[en.col];
                    Ly.entry_q[idx] = en.q;
                    for (int gi = 0; gi < Ga; gi++)
                        Ly.gv[((size_t)gi * CP + c * P + e) * L + lane] =
                            sp.val[(size_t)active[gi] * sp.nnz + en.q];
                }
                part_slots[i].push_back(lane * C + c);
                j++;
            }
        }
    }
    if (nprio) *nprio = most;
    const unsigned zero_part = (unsigned)(L * C) << 16, first = 1u << 31;
    Ly.cw.assign((size_t)kCloseMax * L, (unsigned)(M + 1) | zero_part | first);
    for (int l = 0; l < L; l++) {
        int k = 0;
        for (int i : own[l]) {
            const unsigned row = (unsigned)newpos[i];
            if (part_slots[i].empty()) {
                Ly.cw[(size_t)k++ * L + l] = row | zero_part | first;
                continue;
            }
            for (size_t q = 0; q < part_slots[i].size(); q++)
                Ly.cw[(size_t)k++ * L + l] =
                    row | ((unsigned)part_slots[i][q] << 16) | (q == 0 ? first : 0u);
        }
    }
    Ly.lane_of = own;
    Ly.parts = true;
    Ly.C = C;
    Ly.P = P;
    Ly.kc = bkc;
    Ly.L = L;
    Ly.E = CP;
    Ly.use_reg = false;
    Ly.epl = 0;
    Ly.threads = threads;
    return SSS_OK;
}

// ---------------------------------------------------------------------------
// Slot-packed layout (k_batch_slots with SlotProgram).
//
// Rows are laid lane after lane in lanes of S slots by McNaughton's
// wrap-around rule for preemptive scheduling (McNaughton, Management
// Science 6(1), 1959): a row of n entries takes n + 1 consecutive slots (its
// entries, then its v entry, whose slot stores the row), and a row that
// crosses a lane boundary is cut in two -- its first entries at the start
// of the next lane (a donor, which parks its partial sum) and the rest at
// the end of this lane (a receiver, which starts from that partial sum).
// Donors end by the barrier slot SA = S/2 and receivers start at SA or
// later, so one barrier per Horner term orders them; the cut costs no
// instruction.  A row longer than S first hands entries to standalone
// donors at lane starts (from the last lane back, inside [0, SA)); its own
// piece adds each of their partial sums with one more slot after SA.
// ---------------------------------------------------------------------------
namespace {

struct SlotCell {
    int kind = 0;  // 0 padding, 1 entry, 2 partial add, 3 the row's v entry
    int row = -1, ent = -1, part = -1, pidx = 0;
    int store_row = -1;  // the row this slot's sum completes (stored to the next iterate)
    unsigned flags = 0;
};

bool slots_try(const std::vector<int>& nent, const std::vector<int>& order, int L, int S, int SA,
               std::vector<SlotCell>& cell, int* npart_out) {
    cell.assign((size_t)L * S, SlotCell{});
    auto at = [&](int l, int q) -> SlotCell& { return cell[(size_t)l * S + q]; };
    const bool bar = SA >= 1 && SA < S;
    int npart = 0;
    struct Item { int row, e0, n; std::vector<int> adds; };
    struct Don { int row, e0, n, pidx; };
    std::vector<Item> items;
    std::vector<Don> dons;
    for (int i : order) {
        const int n = nent[i];
        if (n + 1 <= S) {
            items.push_back({i, 0, n, {}});
            continue;
        }
        if (!bar) return false;
        int taken = 0;
        std::vector<int> adds;
        while ((n - taken) + (int)adds.size() + 1 > S) {
            const int k = std::min(SA, n - taken);
            if (k <= 0) return false;
            dons.push_back({i, taken, k, npart});
            adds.push_back(npart++);
            taken += k;
        }
        items.push_back({i, taken, n - taken, adds});
    }
    auto put_donor = [&](int row, int e0, int n, int l, int q0, int pidx) {
        for (int k = 0; k < n; k++) {
            SlotCell& c = at(l, q0 + k);
            c.kind = 1;
            c.row = row;
            c.ent = e0 + k;
            if (k == 0) c.flags |= kSlotStart;
            if (k == n - 1) {
                c.flags |= kSlotDend;
                c.pidx = pidx;
            }
        }
    };
    auto put_closer = [&](int row, int e0, int n, const std::vector<int>& adds, int l, int q0,
                          int recv) {
        int q = q0;
        for (int k = 0; k < n; k++, q++) {
            SlotCell& c = at(l, q);
            c.kind = 1;
            c.row = row;
            c.ent = e0 + k;
        }
        for (int pa : adds) {
            SlotCell& c = at(l, q++);
            c.kind = 2;
            c.row = row;
            c.part = pa;
        }
        SlotCell& c = at(l, q);
        c.kind = 3;
        c.row = row;
        c.store_row = row;
        SlotCell& f = at(l, q0);
        f.flags |= kSlotStart;
        if (recv >= 0) {
            f.flags |= kSlotRecv;
            f.pidx = recv;
        }
    };
    std::vector<int> reserve(L, 0);
    {
        int l = L - 1;
        for (const Don& d : dons) {
            while (l >= 0 && reserve[l] + d.n > SA) l--;
            if (l < 0) return false;
            put_donor(d.row, d.e0, d.n, l, reserve[l], d.pidx);
            reserve[l] += d.n;
        }
    }
    int lane = 0, pos = reserve[0];
    for (const Item& it : items) {
        const int m = (int)it.adds.size();
        const int n = it.n + m + 1;
        while (true) {
            if (lane >= L) return false;
            if (pos + n <= S && (m == 0 || pos + it.n >= SA)) {  // whole, adds after the barrier
                put_closer(it.row, it.e0, it.n, it.adds, lane, pos, -1);
                pos += n;
                if (pos == S) {
                    lane++;
                    pos = lane < L ? reserve[lane] : 0;
                }
                break;
            }
            // cut: receiver [pos, S) here, donor at the start of the next lane
            const int recv_ents = S - pos - 1 - m;
            const int a = it.n - recv_ents;
            if (bar && recv_ents >= 0 && pos >= SA && a >= 1 && lane + 1 < L &&
                reserve[lane + 1] + a <= SA) {
                const int pidx = npart++;
                put_closer(it.row, it.e0 + a, recv_ents, it.adds, lane, pos, pidx);
                put_donor(it.row, it.e0, a, lane + 1, reserve[lane + 1], pidx);
                lane++;
                pos = reserve[lane] + a;
                break;
            }
            lane++;  // pad the rest of this lane
            pos = lane < L ? reserve[lane] : 0;
        }
    }
    *npart_out = npart;
    return true;
}

// Smallest compiled S (up to S_cap) with a slot layout of rows of nent
// entries on L lanes: S from the lower bound ceil(sum(n+1)/L) up, with no cut
// first, then the barrier at S/2, each with the rows in decreasing size and
// then in seeded random orders; the first layout that fits wins.
bool slots_pack(const std::vector<int>& nent, int L, int S_cap, std::vector<SlotCell>& cell,
                int* S_out, int* SA_out, int* npart_out) {
    const int M = (int)nent.size();
    long total = 0;
    for (int n : nent) total += n + 1;
    const int lo = (int)std::max<long>(1, (total + L - 1) / L);
    std::vector<int> base(M);
    std::iota(base.begin(), base.end(), 0);
    std::stable_sort(base.begin(), base.end(), [&](int x, int y) { return nent[x] > nent[y]; });
    const int tries = std::max(8, std::min(4000, 60000 / std::max(1, M)));
    for (int s = lo; s <= std::min(S_cap, kSlotsMax); s++) {
        if (!slot_size_compiled(s)) continue;
        for (int sa : {s, s / 2}) {
            if (sa < 1) continue;
            std::mt19937 rng(1234567u + 31u * s + sa);
            std::vector<int> ord = base;
            for (int t = 0; t < (sa == s ? 2 : tries); t++) {
                if (t > 0) std::shuffle(ord.begin(), ord.end(), rng);
                int np = 0;
                if (slots_try(nent, ord, L, s, sa, cell, &np) && np < (1 << (32 - kSlotPidxShift))) {
                    *S_out = s;
                    *SA_out = sa;
                    *npart_out = np;
                    return true;
                }
            }
        }
    }
    return false;
}

// Phased row-part layout (k_batch_slots with PhasedProgram).  A row of n
// entries is n + 1 items (its entries and its v entry).  Per lane, phase 1
// runs C1 chains of P1 slots and phase 2 runs C2 chains of P2 slots; every
// chain starts at a fixed slot (phase 1 from zero, phase 2 from a parked
// partial sum or zero), so no lane needs a per-slot choice of start value.
// A row is one of
//   * one phase-1 chain (n + 1 <= P1), which stores the row;
//   * one phase-2 chain (n + 1 <= P2), from zero;
//   * k phase-1 chains (parts) and one phase-2 chain that starts from the
//     first part's partial sum, adds the other k - 1 partial sums (one slot
//     each) and the r items left, (k - 1) + r <= P2.
// Rows take the option with the fewest phase-1 chains; chains are dealt to
// lanes round-robin.  items[i] lists row i's items in the order they are
// dealt (entry indices, -1 for the v entry): the first n + 1 - r go to the
// parts round-robin, so items early in the list sit at the lowest chain
// positions of every part, and the last r to the phase-2 chain.
bool phased_pack(const std::vector<int>& nent, const std::vector<std::vector<int>>& items, int L,
                 const PhasedShape& sh, std::vector<SlotCell>& cell, int* npart_out) {
    const int M = (int)nent.size();
    const int C1 = sh.C1, P1 = sh.P1, C2 = sh.C2, P2 = sh.P2;
    const int S1 = C1 * P1, S = S1 + C2 * P2;
    cell.assign((size_t)L * S, SlotCell{});
    struct Choice { int k, r; };
    std::vector<Choice> plan(M);
    long n1 = 0, n2 = 0;
    for (int i = 0; i < M; i++) {
        const int n = nent[i] + 1;
        if (n <= P1) {
            plan[i] = {1, 0};
            n1 += 1;
            continue;
        }
        if (n <= P2) {
            plan[i] = {0, n};
            n2 += 1;
            continue;
        }
        int k = 1;
        for (;; k++) {
            const int rmax = P2 - (k - 1);
            if (rmax < 0) return false;
            if (n - rmax <= k * P1) break;
        }
        plan[i] = {k, std::max(0, n - k * P1)};
        n1 += k;
        n2 += 1;
    }
    if (n1 > (long)C1 * L || n2 > (long)C2 * L) return false;
    auto at = [&](int l, int q) -> SlotCell& { return cell[(size_t)l * S + q]; };
    auto put_item = [&](SlotCell& c, int row, int it) {
        const int e = items[row][it];
        c.row = row;
        if (e >= 0) {
            c.kind = 1;
            c.ent = e;
        } else {
            c.kind = 3;
        }
    };
    int j1 = 0, j2 = 0, npart = 0;
    for (int i = 0; i < M; i++) {
        const Choice& pl = plan[i];
        const int n = nent[i] + 1;
        const bool single = pl.k == 1 && pl.r == 0;
        const int in_parts = n - pl.r;
        int it = in_parts;
        std::vector<int> parts;
        for (int k = 0; k < pl.k; k++) {
            const int lane = j1 % L, ch = j1 / L;
            j1++;
            // part k takes items k, k + pl.k, k + 2 pl.k, ... of the first in_parts
            for (int e = 0, x = k; x < in_parts; e++, x += pl.k) {
                if (e >= P1) return false;
                put_item(at(lane, e * C1 + ch), i, x);
            }
            SlotCell& last = at(lane, (P1 - 1) * C1 + ch);
            if (single) {
                last.store_row = i;
            } else {
                last.flags |= kSlotDend;
                last.pidx = npart;
                parts.push_back(npart++);
            }
        }
        if (single) continue;
        const int lane = j2 % L, ch = j2 / L;
        j2++;
        int e = 0;
        if (!parts.empty()) {
            SlotCell& f = at(lane, S1 + ch);
            f.flags |= kSlotRecv;
            f.pidx = parts[0];
        }
        for (size_t pp = 1; pp < parts.size(); pp++, e++) {
            SlotCell& c = at(lane, S1 + e * C2 + ch);
            c.kind = 2;
            c.row = i;
            c.part = parts[pp];
        }
        for (; it < n; it++, e++) {
            if (e >= P2) return false;
            put_item(at(lane, S1 + e * C2 + ch), i, it);
        }
        at(lane, S1 + (P2 - 1) * C2 + ch).store_row = i;
    }
    *npart_out = npart;
    return true;
}

}  // namespace

// Kernel tables of a slot-cell layout (S slots x L lanes, cell [l*S + q]):
// rows owned by the lane that stores them, renumbered in lane order; load
// words [q][l], then store words [S + q][l] (partial sum p lives at row
// M+2+p of the next iterate); generator values and entry indices per slot
// (entry_q -2 marks a partial add, an entry of coefficient 1).
static int emit_slot_cells(sss_plan* p, const std::vector<std::vector<BatchLayout::Ent>>& rows,
                           const std::vector<SlotCell>& cell, int L, int S, int npart,
                           const std::vector<int>& active, const std::vector<int>& rows_reached,
                           BatchLayout& Ly) {
    const SparseGenerators& sp = p->sparse;
    const int M = (int)rows.size(), Ga = (int)active.size();
    std::vector<std::vector<int>> own(L);
    for (int l = 0; l < L; l++)
        for (int q = 0; q < S; q++)
            if (cell[(size_t)l * S + q].store_row >= 0) own[l].push_back(cell[(size_t)l * S + q].store_row);
    for (auto& o : own) std::sort(o.begin(), o.end());
    std::vector<int>& newpos = Ly.newpos;
    std::vector<int>& row_orig = Ly.row_orig;
    newpos.assign(M, -1);
    row_orig.assign(M, 0);
    {
        int k = 0;
        for (int l = 0; l < L; l++)
            for (int i : own[l]) {
                if (newpos[i] >= 0) return fail(SSS_EINVAL, "slot layout stores a row twice");
                newpos[i] = k;
                row_orig[k] = rows_reached[i];
                k++;
            }
        if (k != M) return fail(SSS_EINVAL, "slot layout lost a row");
    }
    if (M + 2 + npart > (int)kSlotIdx)
        return fail(SSS_EINVAL, "slot layout: rows plus partial sums exceed 16381");
    const unsigned zero_row = (unsigned)M, sink = (unsigned)M + 1;
    Ly.cw.assign((size_t)2 * S * L, 0u);
    Ly.entry_q.assign((size_t)S * L, -1);
    Ly.cval.assign((size_t)S * L, 0.0);
    Ly.gv.assign((size_t)Ga * S * L, 0.0);
    for (int l = 0; l < L; l++)
        for (int q = 0; q < S; q++) {
            const SlotCell& c = cell[(size_t)l * S + q];
            const size_t idx = (size_t)q * L + l;
            unsigned ld = zero_row, st = sink, base = zero_row;
            if (c.kind == 1) {
                const BatchLayout::Ent& en = rows[c.row][c.ent];
                ld = (unsigned)newpos[en.col];
                if (en.q >= sp.nnz) {  // a constant entry
                    Ly.entry_q[idx] = -3;
                    Ly.cval[idx] = p->slot_consts[(size_t)(en.q - sp.nnz)];
                } else {
                    Ly.entry_q[idx] = en.q;
                    for (int gi = 0; gi < Ga; gi++)
                        Ly.gv[((size_t)gi * S + q) * L + l] = sp.val[(size_t)active[gi] * sp.nnz + en.q];
                }
            } else if (c.kind == 2) {
                ld = kLdNext | (unsigned)(M + 2 + c.part);
                Ly.entry_q[idx] = -2;
            } else if (c.kind == 3) {
                ld = kLdV | (unsigned)newpos[c.row];
            }
            if (c.store_row >= 0) st = (unsigned)newpos[c.store_row];
            if (c.flags & kSlotDend) st = (unsigned)(M + 2 + c.pidx);
            if (c.flags & kSlotRecv) base = (unsigned)(M + 2 + c.pidx);
            const bool start = c.kind == 0 || (c.flags & kSlotStart);
            Ly.cw[idx] = ld;
            Ly.cw[(size_t)S * L + idx] = st | (base << 14) | (start ? kStStart : 0u);
        }
    Ly.pcol.clear();
    Ly.lane_of = own;
    return SSS_OK;
}

// Places the rows, parked partial sums and piece items of a slot-programmed
// layout for few shared-memory bank conflicts (optimise_banks) and pads the
// buffer stride M + 2 + npart to a multiple of 16 words, so that word i of
// V, A and B falls in the same bank.  The accesses of one Horner term:
// every slot's operand load, the reloads of parked partial sums after the
// barrier, the loads of phase-2 start values and every store.  Items move
// only inside their piece (or chain) and only among their kind: entries
// of generators assembled every exponential (varies[g]) among themselves,
// so the assembly touches the same slots; other entries and v terms among
// themselves; partial adds stay (they must follow the barrier).  Rewrites
// the kernel words, entry indices, generator values, newpos, row_orig and
// the lanes' row ranges (an even split: the kernels' per-row loops sit
// between group barriers, so any partition of the rows serves).
static int bank_relabel(sss_plan* p, BatchLayout& Ly, const std::vector<int>& active,
                        const std::vector<char>& varies) {
    const int L = Ly.L, S = Ly.S, M = Ly.M, np = Ly.npart, Ga = (int)active.size();
    const int sink = M + 1, n_items = M + 2 + np, bar = Ly.bar_at;
    std::vector<unsigned>& cw = Ly.cw;
    auto ldw = [&](int q, int l) { return cw[(size_t)q * L + l]; };
    auto stw = [&](int q, int l) { return cw[(size_t)(S + q) * L + l]; };
    BankProblem pb;
    pb.L = L;
    auto buf_of = [](unsigned w) {
        const unsigned src = w & (3u << 14);
        return src == kLdV ? 0 : (src == kLdNext ? 2 : 1);
    };
    // instructions: the S operand loads first (cell q*L + l), then the
    // reloads of partial sums after the barrier, start-value loads and stores
    auto instr = [&](auto fn) {  // fn(l) -> access
        for (int l = 0; l < L; l++) pb.cell.push_back(fn(l));
        pb.n_instr++;
    };
    for (int q = 0; q < S; q++)
        instr([&, q](int l) { return BankAccess{buf_of(ldw(q, l)), (int)(ldw(q, l) & kSlotIdx)}; });
    for (int q = bar; q < S; q++)
        instr([&, q](int l) {
            const unsigned w = ldw(q, l);
            return (w & (3u << 14)) == kLdNext ? BankAccess{2, (int)(w & kSlotIdx)} : BankAccess{-1, 0};
        });
    auto add_store = [&](int q) {
        instr([&, q](int l) {
            const int st = (int)(stw(q, l) & kSlotIdx);
            return st == sink ? BankAccess{-1, 0} : BankAccess{2, st};
        });
    };
    auto add_base = [&](int q) {
        instr([&, q](int l) { return BankAccess{2, (int)((stw(q, l) >> 14) & kSlotIdx)}; });
    };
    // pieces (slot-packed: from a start slot to a storing slot) or chains
    // (phased), as lists of load cells per lane
    std::vector<std::vector<int>> pieces;
    if (Ly.phased) {
        const PhasedShape& sh = kPhasedShapes[Ly.shape];
        const int S1 = sh.C1 * sh.P1;
        for (int c = 0; c < sh.C1; c++) add_store((sh.P1 - 1) * sh.C1 + c);
        for (int c = 0; c < sh.C2; c++) {
            add_base(S1 + c);
            add_store(S1 + (sh.P2 - 1) * sh.C2 + c);
        }
        for (int l = 0; l < L; l++) {
            for (int c = 0; c < sh.C1; c++) {
                pieces.emplace_back();
                for (int e = 0; e < sh.P1; e++) pieces.back().push_back((e * sh.C1 + c) * L + l);
            }
            for (int c = 0; c < sh.C2; c++) {
                pieces.emplace_back();
                for (int e = 0; e < sh.P2; e++) pieces.back().push_back((S1 + e * sh.C2 + c) * L + l);
            }
        }
    } else {
        for (int q = 0; q < S; q++) {
            add_store(q);
            if (q >= bar) add_base(q);
        }
        for (int l = 0; l < L; l++) {
            std::vector<int> cur;
            for (int q = 0; q < S; q++) {
                if ((stw(q, l) & kStStart) && !cur.empty()) {
                    pieces.push_back(cur);
                    cur.clear();
                }
                cur.push_back(q * L + l);
                if ((int)(stw(q, l) & kSlotIdx) != sink) {
                    pieces.push_back(cur);
                    cur.clear();
                }
            }
            if (!cur.empty()) pieces.push_back(cur);
        }
    }
    for (const auto& pc : pieces) {
        std::vector<int> var, other;
        for (int c : pc) {
            const int q = c / L, l = c % L;
            const unsigned w = ldw(q, l);
            if ((w & (3u << 14)) == kLdNext) continue;  // partial adds stay
            bool v = false;
            for (int gi = 0; gi < Ga && !v; gi++)
                v = active[gi] < (int)varies.size() && varies[active[gi]] &&
                    Ly.gv[((size_t)gi * S + q) * L + l] != 0.0;
            (v ? var : other).push_back(c);
        }
        if (var.size() >= 2) pb.cell_sets.push_back(var);
        if (other.size() >= 2) pb.cell_sets.push_back(other);
    }
    for (const BankAccess& a : pb.cell)
        if (a.buf >= 0 && (a.item < 0 || a.item >= n_items))
            return fail(SSS_EINVAL, "slot word out of range");
    pb.classes.resize(2);
    for (int i = 0; i < M; i++) pb.classes[0].push_back(i);
    for (int i = M + 2; i < n_items; i++) pb.classes[1].push_back(i);
    // cached per layout (FNV-1a over the kernel words and the item kinds)
    uint64_t key = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { key = (key ^ v) * 1099511628211ull; };
    for (uint64_t v : {(uint64_t)L, (uint64_t)S, (uint64_t)M, (uint64_t)np, (uint64_t)Ly.phased,
                       (uint64_t)Ly.shape, (uint64_t)bar})
        mix(v);
    for (unsigned w : cw) mix(w);
    for (const auto& cs : pb.cell_sets) {
        mix(0xffffffffull);
        for (int c : cs) mix((uint64_t)c);
    }
    std::vector<int> pos(n_items), origin;
    for (int i = 0; i < n_items; i++) pos[i] = i;
    int before = 0, after = 0;
    const int n_load = S * L;
    auto hit = p->bank_cache.find(key);
    if (hit != p->bank_cache.end() && (int)hit->second.size() == n_items + n_load) {
        before = bank_total_cost(pb, pos);
        pos.assign(hit->second.begin(), hit->second.begin() + n_items);
        origin.assign(hit->second.begin() + n_items, hit->second.end());
        std::vector<BankAccess> moved(pb.cell);
        for (int c = 0; c < n_load; c++) moved[c] = pb.cell[origin[c]];
        pb.cell = moved;
        after = bank_total_cost(pb, pos);
    } else {
        // at most a few seconds of host time, once per layout (NV-21's
        // 249 labels: about 2.5 s; NV-7 converges in a fraction of that)
        const long budget = std::min<long>(20000000L, 300000L + 80000L * (long)(M + np));
        after = optimise_banks(pb, pos, origin, budget, &before);
        origin.resize(n_load);
        std::vector<int> entry(pos);
        entry.insert(entry.end(), origin.begin(), origin.end());
        p->bank_cache[key] = entry;
    }
    p->last_bank_before = before;
    p->last_bank_after = after;
    // rewrite: items moved within lanes (load words, entry indices,
    // generator values), then every word relabelled
    {
        const std::vector<unsigned> cw0(cw);
        const std::vector<int> eq0(Ly.entry_q);
        const std::vector<double> gv0(Ly.gv), cv0(Ly.cval);
        for (int c = 0; c < n_load; c++) {
            const int o = origin[c];
            if (o == c) continue;
            const int q = c / L, l = c % L, qo = o / L;
            cw[(size_t)q * L + l] = cw0[(size_t)qo * L + l];
            Ly.entry_q[(size_t)q * L + l] = eq0[(size_t)qo * L + l];
            if (!cv0.empty()) Ly.cval[(size_t)q * L + l] = cv0[(size_t)qo * L + l];
            for (int gi = 0; gi < Ga; gi++)
                Ly.gv[((size_t)gi * S + q) * L + l] = gv0[((size_t)gi * S + qo) * L + l];
        }
    }
    for (int q = 0; q < S; q++)
        for (int l = 0; l < L; l++) {
            unsigned& w = cw[(size_t)q * L + l];
            w = (w & ~kSlotIdx) | (unsigned)pos[w & kSlotIdx];
            unsigned& s2 = cw[(size_t)(S + q) * L + l];
            const unsigned st = s2 & kSlotIdx, base = (s2 >> 14) & kSlotIdx;
            s2 = (s2 & ~(kSlotIdx | (kSlotIdx << 14))) | (unsigned)pos[st] |
                 ((unsigned)pos[base] << 14);
        }
    std::vector<int> row_orig(M), inv(M);
    for (int k = 0; k < M; k++) row_orig[pos[k]] = Ly.row_orig[k];
    Ly.row_orig = row_orig;
    for (int& r : Ly.newpos)
        if (r >= 0) r = pos[r];
    for (int i = 0; i < (int)Ly.newpos.size(); i++)
        if (Ly.newpos[i] >= 0) inv[Ly.newpos[i]] = i;
    Ly.lane_of.assign(L, {});
    for (int l = 0; l < L; l++)
        for (int k = (int)((long)M * l / L); k < (int)((long)M * (l + 1) / L); k++)
            Ly.lane_of[l].push_back(inv[k]);
    Ly.npart = (M + 2 + np + 15) / 16 * 16 - (M + 2);
    return SSS_OK;
}

int place_banks(sss_plan* p, BatchLayout& Ly, const std::vector<int>& active,
                const std::vector<char>& varies) {
    return bank_relabel(p, Ly, active, varies);
}

static void set_slot_fields(BatchLayout& Ly, int L, int S, int SA, int npart, int threads) {
    Ly.parts = true;
    Ly.slots = true;
    Ly.C = 1;
    Ly.P = S;
    Ly.kc = 0;
    Ly.S = S;
    Ly.bar_at = SA;
    Ly.npart = npart;
    Ly.L = L;
    Ly.E = S;
    Ly.use_reg = false;
    Ly.epl = 0;
    Ly.threads = threads;
}

// Slot-packed layout at L lanes with at most S_cap slots; SSS_EINVAL when
// none fits.
int slots_layout_rows(sss_plan* p, const std::vector<std::vector<BatchLayout::Ent>>& rows, int L,
                      int threads, int S_cap, const std::vector<int>& active,
                      const std::vector<int>& rows_reached, BatchLayout* out) {
    BatchLayout& Ly = *out;
    const int M = (int)rows.size();
    if (L != 8 && L != 16 && L != 32 && L != 64 && L != 128 && L != 256)
        return fail(SSS_EINVAL, "slot-packed variant needs 8 to 256 lanes per trajectory (a power of two)");
    if (L > 32) threads = L;
    if (threads % L) return fail(SSS_EINVAL, "CTA size must be a multiple of the lanes per trajectory");
    if (M + 2 > (int)kSlotIdx) return fail(SSS_EINVAL, "slot-packed variant supports at most 16381 rows");
    std::vector<int> nent(M);
    for (int i = 0; i < M; i++) nent[i] = (int)rows[i].size();
    std::vector<SlotCell> cell;
    int S = 0, SA = 0, npart = 0;
    if (!slots_pack(nent, L, S_cap, cell, &S, &SA, &npart))
        return fail(SSS_EINVAL, "slot-packed variant does not fit this pattern at " + std::to_string(L) +
                                    " lanes per trajectory");
    if (int rc = emit_slot_cells(p, rows, cell, L, S, npart, active, rows_reached, Ly)) return rc;
    set_slot_fields(Ly, L, S, SA, npart, threads);
    Ly.phased = false;
    return SSS_OK;
}

// Phased row-part layout at L lanes: the first shape of kPhasedShapes (in
// order of slots per lane, at most S_cap) that fits.
// varies[g] (per generator slot, may be empty): its coefficient varies, so
// its entries are assembled every exponential.
int phased_layout_rows(sss_plan* p, const std::vector<std::vector<BatchLayout::Ent>>& rows, int L,
                       int threads, int S_cap, const std::vector<int>& active,
                       const std::vector<int>& rows_reached, const std::vector<char>& varies,
                       BatchLayout* out) {
    BatchLayout& Ly = *out;
    const int M = (int)rows.size();
    // the forward kernels compile phased programs for warp groups (8-32
    // lanes); the adjoint's block series also for 64-lane groups
    if (L != 8 && L != 16 && L != 32 && L != 64)
        return fail(SSS_EINVAL, "phased row-part variant needs 8, 16, 32 or 64 lanes per trajectory");
    if (L > 32) threads = L;  // a group wider than a warp is one CTA
    if (threads % L) return fail(SSS_EINVAL, "CTA size must be a multiple of the lanes per trajectory");
    if (M + 2 > (int)kSlotIdx) return fail(SSS_EINVAL, "phased row-part variant supports at most 16381 rows");
    std::vector<int> nent(M);
    for (int i = 0; i < M; i++) nent[i] = (int)rows[i].size();
    // item order per row: entries of generators whose coefficient varies
    // (assembled every exponential) first, then the others, then the v
    // entry, so the varying entries of every chain sit at its first slots
    // and the per-exponential assembly touches few slot positions
    const SparseGenerators& sp = p->sparse;
    std::vector<std::vector<int>> items(M);
    for (int i = 0; i < M; i++) {
        std::vector<int> later;
        for (int e = 0; e < nent[i]; e++) {
            bool var = false;
            for (int g : active)
                var |= rows[i][e].q < sp.nnz && g < (int)varies.size() && varies[g] &&
                       sp.val[(size_t)g * sp.nnz + rows[i][e].q] != 0.0;
            (var ? items[i] : later).push_back(e);
        }
        items[i].insert(items[i].end(), later.begin(), later.end());
        items[i].push_back(-1);
    }
    std::vector<SlotCell> cell;
    int best = -1, npart = 0;
    for (int k = 0; k < kPhasedShapeCount && best < 0; k++) {
        const PhasedShape& sh = kPhasedShapes[k];
        if (sh.C1 * sh.P1 + sh.C2 * sh.P2 > S_cap) continue;
        if (phased_pack(nent, items, L, sh, cell, &npart)) best = k;
    }
    if (best < 0)
        return fail(SSS_EINVAL, "phased row-part variant does not fit this pattern at " +
                                    std::to_string(L) + " lanes per trajectory");
    const PhasedShape& sh = kPhasedShapes[best];
    const int S = sh.C1 * sh.P1 + sh.C2 * sh.P2;
    if (int rc = emit_slot_cells(p, rows, cell, L, S, npart, active, rows_reached, Ly)) return rc;
    set_slot_fields(Ly, L, S, sh.C1 * sh.P1, npart, threads);
    Ly.phased = true;
    Ly.shape = best;
    return SSS_OK;
}

// Per column of a coefficient table (rows x G): the largest |value|, the
// smallest and largest value, and a count of non-finite values; one partial
// per CTA in out[(cta*G + g)*4 + {0,1,2,3}], reduced on the host.
__global__ void __launch_bounds__(256) k_table_stats(const double* __restrict__ tab, size_t rows,
                                                     int G, double* __restrict__ out) {
    __shared__ double s_red[8][kMaxG][4];
    double st[kMaxG][4];
    for (int g = 0; g < kMaxG; g++) {
        st[g][0] = 0.0;
        st[g][1] = INFINITY;
        st[g][2] = -INFINITY;
        st[g][3] = 0.0;
    }
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += (size_t)gridDim.x * blockDim.x)
        for (int g = 0; g < G; g++) {
            const double v = __ldg(tab + r * G + g);
            if (!isfinite(v)) {
                st[g][3] += 1.0;
            } else {
                st[g][0] = fmax(st[g][0], fabs(v));
                st[g][1] = fmin(st[g][1], v);
                st[g][2] = fmax(st[g][2], v);
            }
        }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int g = 0; g < G; g++)
        for (int o = 16; o > 0; o >>= 1) {
            st[g][0] = fmax(st[g][0], __shfl_xor_sync(0xffffffffu, st[g][0], o));
            st[g][1] = fmin(st[g][1], __shfl_xor_sync(0xffffffffu, st[g][1], o));
            st[g][2] = fmax(st[g][2], __shfl_xor_sync(0xffffffffu, st[g][2], o));
            st[g][3] += __shfl_xor_sync(0xffffffffu, st[g][3], o);
        }
    if (lane == 0)
        for (int g = 0; g < G; g++)
            for (int j = 0; j < 4; j++) s_red[warp][g][j] = st[g][j];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            for (int g = 0; g < G; g++) {
                s_red[0][g][0] = fmax(s_red[0][g][0], s_red[w][g][0]);
                s_red[0][g][1] = fmin(s_red[0][g][1], s_red[w][g][1]);
                s_red[0][g][2] = fmax(s_red[0][g][2], s_red[w][g][2]);
                s_red[0][g][3] += s_red[w][g][3];
            }
        for (int g = 0; g < G; g++)
            for (int j = 0; j < 4; j++) out[((size_t)blockIdx.x * G + g) * 4 + j] = s_red[0][g][j];
    }
}

// Column statistics of a device coefficient table: the channels' bounds
// and which channels hold one value everywhere (folded into the constant
// part of Omega).  A NaN or infinite entry is an error.
static int table_stats(sss_plan* p, const double* d_tab, size_t rows, int G, std::vector<double>& chmax,
                       std::vector<double>& chval, std::vector<char>& chconst, cudaStream_t st) {
    const int threads = 256;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((rows + threads - 1) / threads,
                                                                 (size_t)2 * p->num_sms));
    if (int rc = p->w_status.ensure(sizeof(double) * (size_t)blocks * G * 4)) return rc;
    k_table_stats<<<blocks, threads, 0, st>>>(d_tab, rows, G, p->w_status.as<double>());
    SSS_CUDA(cudaGetLastError());
    std::vector<double> part((size_t)blocks * G * 4);
    SSS_CUDA(cudaMemcpyAsync(part.data(), p->w_status.p, sizeof(double) * part.size(),
                             cudaMemcpyDeviceToHost, st));
    SSS_CUDA(cudaStreamSynchronize(st));
    for (int g = 0; g < G; g++) {
        double mx = 0.0, lo = INFINITY, hi = -INFINITY, bad = 0.0;
        for (int c = 0; c < blocks; c++) {
            const double* q = &part[((size_t)c * G + g) * 4];
            mx = std::max(mx, q[0]);
            lo = std::min(lo, q[1]);
            hi = std::max(hi, q[2]);
            bad += q[3];
        }
        if (bad > 0.0)
            return fail(SSS_ENONFINITE, "coefficient table column " + std::to_string(g) +
                                            " contains NaN or infinity");
        chmax[g] = mx;
        chconst[g] = rows > 0 && lo == hi;
        chval[g] = rows > 0 ? lo : 0.0;
    }
    return SSS_OK;
}

// FP64 instructions per Horner term of one group: C*P + kc for the row-part
// layout, S for the slot-packed and phased ones; a group wider than a warp
// pays about half an instruction per CTA barrier.
static double layout_cost(const BatchLayout& Ly) {
    double c = Ly.slots ? Ly.S : Ly.C * Ly.P + Ly.kc;
    if (Ly.L > 32) c += 0.5 * (Ly.slots ? (Ly.bar_at < Ly.S ? 2 : 1) : 2);
    return c;
}

// Automatic lane count for n trajectories (auto_lane_count on this GPU's
// sub-partitions) from the cost of the best layout at each lane count 8,
// 16, ..., 256 (0: does not fit).  0 when nothing fits.
int auto_lanes(const sss_plan* p, const double* cost, long n) {
    return auto_lane_count(4L * p->num_sms, cost, n);
}

int build_layout(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg,
                 const double* d_prog, double dt, int F, const std::vector<int>& force_active,
                 bool allow_register, BatchLayout* out, cudaStream_t st, bool force_parts,
                 const double* d_tab, int T_tab) {
    const int N = p->d.N;
    const bool rot = p->rotating;
    const bool table = d_tab != nullptr;
    BatchLayout& Ly = *out;
    const SparseGenerators& sp = p->sparse;
    const int G = sp.G;  // generator slots: lab generators, or rotating (node, generator)
    // channel of a slot.  Programs: lab slot g is driven by channel g-1 (slot
    // 0, L0, has coefficient 1); rotating slot k*G0 + g by channel g.  A
    // coefficient table: the slot's column (lab g, rotating g of node k).
    if (table) {
        nch = p->d.G;
        nseg = 0;
    }
    auto slot_chan = [&](int a) { return rot ? a % p->d.G : (table ? a : a - 1); };
    std::vector<double> h_rho0((size_t)ntraj * N), h_prog((size_t)ntraj * nch * nseg * 5);
    SSS_CUDA(cudaMemcpyAsync(h_rho0.data(), d_rho0, sizeof(double) * h_rho0.size(),
                             cudaMemcpyDeviceToHost, st));
    if (!h_prog.empty())
        SSS_CUDA(cudaMemcpyAsync(h_prog.data(), d_prog, sizeof(double) * h_prog.size(),
                                 cudaMemcpyDeviceToHost, st));
    SSS_CUDA(cudaStreamSynchronize(st));
    // ---- channels: largest |coefficient|, and whether the channel holds one
    // constant value for every trajectory at all times (every segment of
    // zero amplitude with the same offset, the last one never ending; or
    // one value in the whole table column): the row-part kernel folds those
    // into the constant part of Omega ----
    std::vector<double> chmax(std::max(nch, 1), 0.0), chval(std::max(nch, 1), 0.0);
    std::vector<char> chconst(std::max(nch, 1), 0);
    if (table) {
        const size_t rows = (size_t)ntraj * F * T_tab * p->d.Q;
        if (int rc = table_stats(p, d_tab, rows, nch, chmax, chval, chconst, st)) return rc;
    }
    for (int c = 0; c < nch && !table; c++) {
        bool ok = ntraj > 0 && nseg > 0;
        double val = 0.0;
        for (int b = 0; b < ntraj; b++) {
            const double* seg = &h_prog[((size_t)b * nch + c) * nseg * 5];
            if (!(seg[(size_t)(nseg - 1) * 5] == INFINITY)) ok = false;
            for (int q = 0; q < nseg; q++) {
                const double* sq = seg + (size_t)q * 5;
                if (sq[0] != -INFINITY)  // a segment that can match
                    chmax[c] = std::max(chmax[c], std::fabs(sq[1]) + std::fabs(sq[2]));
                if (!ok) continue;
                if (sq[2] != 0.0 || !(sq[1] == sq[1])) ok = false;
                else if (b == 0 && q == 0) val = sq[1];
                else if (sq[1] != val) ok = false;
            }
        }
        chconst[c] = ok;
        chval[c] = val;
    }
    std::vector<double> cmax(G, 0.0);
    Ly.chan_const.assign(G, 0);
    Ly.chan_value.assign(G, 0.0);
    Ly.slot_chan.assign(G, -1);
    for (int a = 0; a < G; a++) {
        const int c = slot_chan(a);
        Ly.slot_chan[a] = c;
        if (c < 0) {
            cmax[a] = 1.0;
        } else if (c < nch) {
            cmax[a] = chmax[c];
            Ly.chan_const[a] = chconst[c];
            Ly.chan_value[a] = chval[c];
        }
    }
    std::vector<int> active;
    for (int g = 0; g < G; g++) {
        bool nonzero_gen = false;
        for (int q = 0; q < sp.nnz; q++) nonzero_gen |= sp.val[(size_t)g * sp.nnz + q] != 0.0;
        bool forced = std::find(force_active.begin(), force_active.end(), g) != force_active.end();
        if ((cmax[g] > 0.0 || forced) && nonzero_gen) active.push_back(g);
    }
    const int Ga = (int)active.size();
    // ---- reachable rows from the initial states' support (in the eigenbasis
    // for a rotating plan: the entries of V^-1 rho0 above 1e-15 of its
    // largest), closed under the pattern and, rotating, the e^{L0 h} pairs ----
    std::vector<char> reach(N, 0);
    std::vector<int> stack;
    for (int b = 0; b < ntraj; b++) {
        const double* r0b = &h_rho0[(size_t)b * N];
        if (rot) {
            std::vector<double> xe(N, 0.0);
            double mx = 0.0;
            for (int i = 0; i < N; i++) {
                double o = 0.0;
                for (int j = 0; j < N; j++) o += p->Vinv[(size_t)i * N + j] * r0b[j];
                xe[i] = o;
                mx = std::max(mx, std::fabs(o));
            }
            for (int i = 0; i < N; i++)
                if (std::fabs(xe[i]) > 1e-15 * mx && !reach[i]) { reach[i] = 1; stack.push_back(i); }
        } else {
            for (int i = 0; i < N; i++)
                if (r0b[i] != 0.0 && !reach[i]) { reach[i] = 1; stack.push_back(i); }
        }
    }
    std::vector<std::vector<int>> influences(N);
    if (rot)
        for (int i = 0; i < 2 * p->D; i++) influences[i].push_back(i ^ 1);
    for (int r = 0; r < N; r++)
        for (int q = sp.row_ptr[r]; q < sp.row_ptr[r + 1]; q++) {
            bool nz = false;
            for (int g : active) nz |= sp.val[(size_t)g * sp.nnz + q] != 0.0;
            if (nz) influences[sp.col[q]].push_back(r);
        }
    while (!stack.empty()) {
        int c = stack.back();
        stack.pop_back();
        for (int r : influences[c])
            if (!reach[r]) { reach[r] = 1; stack.push_back(r); }
    }
    std::vector<int> rows_reached;
    for (int i = 0; i < N; i++)
        if (reach[i]) rows_reached.push_back(i);
    const int M = (int)rows_reached.size();
    Ly.M = M;
    Ly.Ga = Ga;
    Ly.active = active;
    if (M == 0) return SSS_OK;
    if (M > 65534) return fail(SSS_EINVAL, "batched kernel supports at most 65534 reachable rows");
    std::vector<int> pos_of_orig(N, -1);
    for (int k = 0; k < M; k++) pos_of_orig[rows_reached[k]] = k;
    // pruned pattern per reachable row: (compressed col, index into sp.val)
    std::vector<std::vector<BatchLayout::Ent>>& row_ents = Ly.row_ents;
    row_ents.assign(M, {});
    long nnz = 0;
    for (int k = 0; k < M; k++) {
        int r = rows_reached[k];
        for (int q = sp.row_ptr[r]; q < sp.row_ptr[r + 1]; q++) {
            int c = sp.col[q];
            if (!reach[c]) continue;
            bool nz = false;
            for (int g : active) nz |= sp.val[(size_t)g * sp.nnz + q] != 0.0;
            if (!nz) continue;
            row_ents[k].push_back({pos_of_orig[c], q});
            nnz++;
        }
    }

    // ---- norm bound -> Taylor degree and sub-steps ----
    double wsum = 0.0;
    for (int e = 0; e < p->d.K; e++) {
        double s = 0.0;
        for (int k = 0; k < p->d.Q; k++) s += std::fabs(p->W[e * p->d.Q + k]);
        wsum = std::max(wsum, s);
    }
    if (rot) {  // a slot's weight is h W[e,k] c: bound sum_k |W[e,k]| by the largest |W|
        wsum = 0.0;
        for (int i = 0; i < p->d.K * p->d.Q; i++) wsum = std::max(wsum, std::fabs(p->W[i]));
    }
    double beta = 0.0;
    for (int g : active) {
        std::vector<double> colsum(M, 0.0);
        for (int k = 0; k < M; k++)
            for (const BatchLayout::Ent& en : row_ents[k]) colsum[en.col] += std::fabs(sp.val[(size_t)g * sp.nnz + en.q]);
        beta += cmax[g] * *std::max_element(colsum.begin(), colsum.end());
    }
    beta *= wsum * dt / F;
    int degree, substeps;
    choose_taylor(beta, p->d.taylor_degree, &degree, &substeps);

    // ---- lanes per trajectory ----
    // GB300 FP64 (~2 DFMA/clk/SM, 75-cycle latency) wants several warps per
    // SM.  Take the fewest lanes giving ~8 warps per SM, capped by the rows
    // available to split.
    int L = 2;
    {
        const long want = (long)p->num_sms * 8 * 32;
        int cap = 2;
        while (cap < 32 && cap * 2 <= std::max(2, M)) cap *= 2;
        while (L < cap && (long)ntraj * L < want) L *= 2;
    }
    if (p->batch_lanes > 0) L = p->batch_lanes;
    // row-part kernel: asked for (4), or automatic (0) when the pattern fits.
    // Automatic lanes: 32 (one trajectory per warp, the shortest chains)
    // while the batch gives at most two warps per SM sub-partition, else 16
    // (two trajectories per warp, fewer instructions per trajectory)
    const bool parts_asked = p->batch_variant == 4 || p->batch_variant == 5;
    const bool slots_asked = p->batch_variant == 6;
    const bool phased_asked = p->batch_variant == 7;
    const bool row_kernels = parts_asked || slots_asked || phased_asked;
    const bool slots_ok = !force_parts && (p->batch_variant == 0 || slots_asked);
    const bool phased_ok = !force_parts && (p->batch_variant == 0 || phased_asked);
    const bool parts_ok = force_parts || (!slots_asked && !phased_asked);
    if (rot && !force_parts && allow_register && p->batch_variant != 0 && !row_kernels)
        return fail(SSS_EINVAL, "the rotating frame runs on the row-part, slot-packed or phased "
                                "kernel (variant 0, 4, 6 or 7)");
    if (table && !force_parts && p->batch_variant != 0 && !row_kernels)
        return fail(SSS_EINVAL, "a coefficient table runs on the row-part, slot-packed or phased "
                                "kernel (variant 0, 4, 6 or 7)");
    if (force_parts || (allow_register && (rot || table || row_kernels || p->batch_variant == 0))) {
        const int threads_cfg = p->batch_threads > 0 ? p->batch_threads : 32;
        std::vector<char> varies(G, 0);
        for (int g = 0; g < G; g++) varies[g] = Ly.slot_chan[g] >= 0 && !Ly.chan_const[g];
        // At Lc lanes: the cheapest of the row-part (0), phased row-part (1)
        // and slot-packed (2) layouts that fit (FP64 instructions per Horner
        // term, layout_cost); ties go to the earlier one (the phased
        // layout's fixed chain starts beat the slot-packed layout's per-slot
        // start selects at equal slots).  The layout functions write only
        // the layout fields of their output.
        auto best_at = [&](int Lc, bool fill) {
            double cost[3] = {0.0, 0.0, 0.0};
            int cap[3] = {0, 0, 0};
            BatchLayout t;
            if (parts_ok && parts_layout_rows(p, Ly.row_ents, {}, Lc, threads_cfg, 1, 1, active,
                                              rows_reached, &t, nullptr) == SSS_OK)
                cost[0] = layout_cost(t);
            auto cap_below = [](double c) { return c > 0.0 ? (int)std::ceil(c) - 1 : 64; };
            cap[1] = cap_below(cost[0]);
            if (phased_ok && Lc <= 32 && cap[1] >= 1) {
                BatchLayout tq;
                if (phased_layout_rows(p, Ly.row_ents, Lc, threads_cfg, cap[1], active, rows_reached,
                                       varies, &tq) == SSS_OK)
                    cost[1] = layout_cost(tq);
            }
            double lim = 0.0;
            for (double c : {cost[0], cost[1]})
                if (c > 0.0 && (lim == 0.0 || c < lim)) lim = c;
            cap[2] = std::min(kSlotsMax, cap_below(lim));
            if (slots_ok && cap[2] >= 1) {
                BatchLayout ts;
                if (slots_layout_rows(p, Ly.row_ents, Lc, threads_cfg, cap[2], active, rows_reached,
                                      &ts) == SSS_OK)
                    cost[2] = layout_cost(ts);
            }
            int pick = -1;
            for (int k = 0; k < 3; k++)
                if (cost[k] > 0.0 && (pick < 0 || cost[k] < cost[pick])) pick = k;
            if (pick < 0) return 0.0;
            if (fill) {
                int r = SSS_EINVAL;
                if (pick == 0)
                    r = parts_layout_rows(p, Ly.row_ents, {}, Lc, threads_cfg, 1, 1, active,
                                          rows_reached, out, nullptr);
                else if (pick == 1)
                    r = phased_layout_rows(p, Ly.row_ents, Lc, threads_cfg, cap[1], active,
                                           rows_reached, varies, out);
                else
                    r = slots_layout_rows(p, Ly.row_ents, Lc, threads_cfg, cap[2], active,
                                          rows_reached, out);
                if (r != SSS_OK) return 0.0;
            }
            return cost[pick];
        };
        // lanes as configured, or the automatic count (auto_lanes)
        int rc = SSS_EINVAL, chosen = 0;
        if (p->batch_lanes > 0) {
            chosen = L;
        } else {
            const long n_rule = p->auto_lanes_ntraj > 0 ? p->auto_lanes_ntraj : ntraj;
            for (int i = 0; i < kLaneCounts; i++) p->auto_cost[i] = best_at(8 << i, false);
            chosen = auto_lanes(p, p->auto_cost, n_rule);
        }
        if (chosen && best_at(chosen, true) > 0.0) {
            rc = Ly.slots ? bank_relabel(p, Ly, active, varies) : SSS_OK;
        } else {
            const char* what = slots_asked ? "slot-packed" : phased_asked ? "phased row-part" : "row-part";
            rc = chosen ? fail(SSS_EINVAL, std::string(what) + " variant does not fit this pattern at " +
                                               std::to_string(chosen) + " lanes per trajectory")
                        : fail(SSS_EINVAL, std::string(what) + " variant does not fit this pattern");
        }
        if (rc == SSS_OK) {
            Ly.nnz = nnz;
            Ly.degree = degree;
            Ly.substeps = substeps;
        }
        if (rc == SSS_OK || row_kernels || force_parts || rot || table) return rc;
    }
    if (L > 32)
        return fail(SSS_EINVAL, "more than 32 lanes per trajectory needs the row-part variant, "
                                "which does not fit this pattern");
    // ---- rows to lanes, balanced by entry count.  The register variant
    // pads each row to an even length (two chains); an empty row carries
    // zero entries so that it still closes ----
    int epl = 0;
    bool use_reg = false;
    std::vector<std::vector<int>> lane_of;
    auto assign = [&](bool pad2) {
        auto cost = [&row_ents, pad2](int i) {
            int n = std::max<int>(1, (int)row_ents[i].size());
            return pad2 ? ((n + 1) & ~1) : n;
        };
        std::vector<int> order(M);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
        std::vector<long> load(L, 0);
        lane_of.assign(L, {});
        for (int i : order) {
            int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            load[l] += cost(i);
            lane_of[l].push_back(i);
        }
        for (auto& lo : lane_of) std::sort(lo.begin(), lo.end());
        return std::make_pair((int)*std::max_element(load.begin(), load.end()),
                              std::function<int(int)>(cost));
    };
    const bool pad2 = p->batch_variant != 3;
    auto reg_try = assign(pad2);
    if (allow_register && reg_try.first <= 64 && p->batch_variant != 2) {
        use_reg = true;
        epl = 8;
        while (epl < reg_try.first) epl *= 2;
    }
    auto plan_lanes = use_reg ? reg_try : assign(false);
    const std::function<int(int)>& cost = plan_lanes.second;
    const int E = use_reg ? epl : plan_lanes.first;
    const int threads = p->batch_threads > 0 ? p->batch_threads : 64;
    if (threads % L) return fail(SSS_EINVAL, "CTA size must be a multiple of the lanes per trajectory");

    // compressed row index = position in the lane-ordered list
    std::vector<int>& newpos = Ly.newpos;
    std::vector<int>& row_orig = Ly.row_orig;
    newpos.assign(M, 0);
    row_orig.assign(M, 0);
    {
        int k = 0;
        for (int l = 0; l < L; l++)
            for (int i : lane_of[l]) { newpos[i] = k; row_orig[k] = rows_reached[i]; k++; }
    }
    // generator values [g][e][l] and entry words [e][l]
    Ly.gv.assign((size_t)Ga * E * L, 0.0);
    Ly.words.assign((size_t)E * L, 0u);
    Ly.cnt.assign(L, 0);
    Ly.entry_q.assign((size_t)E * L, -1);
    for (int l = 0; l < L; l++) {
        int e = 0;
        for (int i : lane_of[l]) {
            const auto& ents = row_ents[i];
            int n = cost(i);
            for (int j = 0; j < n; j++) {
                int col = j < (int)ents.size() ? ents[j].col : i;
                unsigned w = (unsigned)newpos[col];
                if (j == n - 1) w |= (unsigned)(newpos[i] + 1) << 16;
                Ly.words[(size_t)(e + j) * L + l] = w;
                if (j < (int)ents.size()) {
                    Ly.entry_q[(size_t)(e + j) * L + l] = ents[j].q;
                    for (int gi = 0; gi < Ga; gi++)
                        Ly.gv[((size_t)gi * E + e + j) * L + l] = sp.val[(size_t)active[gi] * sp.nnz + ents[j].q];
                }
            }
            e += n;
        }
        Ly.cnt[l] = e;
    }
    Ly.L = L;
    Ly.E = E;
    Ly.use_reg = use_reg;
    Ly.epl = epl;
    Ly.nnz = nnz;
    Ly.degree = degree;
    Ly.substeps = substeps;
    Ly.threads = threads;
    Ly.lane_of = lane_of;
    return SSS_OK;
}

// Device tables (into `tables`) and kernel arguments of a batch layout;
// `keep_live` generators are never folded into the row-part kernel's
// constant part of Omega.
static int make_args(sss_plan* p, const BatchLayout& Ly, int ntraj, int nch, int nseg, double dt,
                     int F, const double* h_rw, const std::vector<int>& keep_live, DevBuf& tables,
                     BatchArgs* out, size_t* smem, cudaStream_t st) {
    const int M = Ly.M, Ga = Ly.Ga, L = Ly.L, E = Ly.E, degree = Ly.degree,
              substeps = Ly.substeps, threads = Ly.threads;
    const bool use_reg = Ly.use_reg;
    const bool one_chain = p->batch_variant == 3;
    const int N = p->d.N;
    const std::vector<int>& active = Ly.active;
    const std::vector<int>& row_orig = Ly.row_orig;
    const bool rot = p->rotating;
    std::vector<double> rw(M, 0.0);
    if (h_rw) {
        if (rot) {  // readout of V x: weights V^T w on the kept eigenbasis rows
            for (int k = 0; k < M; k++) {
                double o = 0.0;
                for (int i = 0; i < N; i++) o += h_rw[i] * p->V[(size_t)i * N + row_orig[k]];
                rw[k] = o;
            }
        } else {
            for (int k = 0; k < M; k++) rw[k] = h_rw[row_orig[k]];
        }
    }
    std::vector<double> toff(F), noff(p->d.Q);
    for (int r = 0; r < F; r++) toff[r] = ((double)r * dt) / F;
    for (int k = 0; k < p->d.Q; k++) noff[k] = (dt * p->nodes[k]) / F;

    std::vector<double> dbl(Ly.gv);
    const std::vector<unsigned>& words = Ly.parts ? Ly.cw : Ly.words;
    // entries per lane (or part columns), then row_orig
    std::vector<int> ints(Ly.parts ? Ly.pcol : Ly.cnt);
    const size_t n_lane_ints = ints.size();
    // row-part variant: the constant part of Omega per exponential -- L0
    // (coefficient 1 in the lab frame) and the channels that are constant
    // over the batch -- formed as the kernel would (weight sum_k W[e,k]*c, or
    // W[e,k]*c for a rotating slot of node k, times h, times the generator,
    // accumulated by FMA in generator order); the other active generators
    // stay live in the kernel, their channels sampled into the ring
    std::vector<int> live, live_k, live_ch, lch;
    const size_t o_om0 = dbl.size();
    if (Ly.parts) {
        const int CP = Ly.C * Ly.P;
        const double h_sub = dt / F / substeps;
        std::vector<double> om0((size_t)p->d.K * CP * L, 0.0);
        for (int gi = 0; gi < Ga; gi++) {
            const int g = active[gi];
            const int ch = Ly.slot_chan[g];
            const int node = rot ? g / p->d.G : -1;
            const bool keep = std::find(keep_live.begin(), keep_live.end(), g) != keep_live.end();
            if (ch >= 0 && (!Ly.chan_const[g] || keep)) {
                live.push_back(gi);
                live_k.push_back(node);
                int ci = (int)(std::find(lch.begin(), lch.end(), ch) - lch.begin());
                if (ci == (int)lch.size()) lch.push_back(ch);
                live_ch.push_back(ci);
                continue;
            }
            const double X = ch < 0 ? 1.0 : Ly.chan_value[g];
            for (int e = 0; e < p->d.K; e++) {
                double s = 0.0;
                if (node < 0)
                    for (int k = 0; k < p->d.Q; k++) s = std::fma(p->W[e * p->d.Q + k], X, s);
                else
                    s = p->W[e * p->d.Q + node] * X;
                const double ag = s * h_sub;
                for (int i = 0; i < CP * L; i++) {
                    double& o = om0[(size_t)e * CP * L + i];
                    o = std::fma(ag, Ly.gv[(size_t)gi * CP * L + i], o);
                }
            }
        }
        // slot layouts: a partial add is an entry of coefficient 1
        if (Ly.slots)
            for (int e = 0; e < p->d.K; e++)
                for (int i = 0; i < CP * L; i++)
                    if (Ly.entry_q[i] == -2) om0[(size_t)e * CP * L + i] = 1.0;
        dbl.insert(dbl.end(), om0.begin(), om0.end());
    }
    const size_t n_gv = dbl.size();
    dbl.insert(dbl.end(), rw.begin(), rw.end());
    dbl.insert(dbl.end(), toff.begin(), toff.end());
    dbl.insert(dbl.end(), noff.begin(), noff.end());
    // rotating frame: e^{L0 h} per kept row -- its own coefficient (minus 1
    // in residual form, as the plan's tables hold it) and its partner's
    const size_t o_blk = dbl.size();
    std::vector<int> blk_pos;
    if (rot) {
        std::vector<int> pos_of(N, M);
        for (int k = 0; k < M; k++) pos_of[row_orig[k]] = k;
        std::vector<double> bs(M), bp(M, 0.0);
        blk_pos.assign(M, M);
        for (int k = 0; k < M; k++) {
            const int i = row_orig[k];
            if (i < 2 * p->D) {
                const double pp = p->dlast[2 * (i / 2)], qq = p->dlast[2 * (i / 2) + 1];
                bs[k] = pp;
                bp[k] = (i & 1) ? qq : -qq;
                blk_pos[k] = pos_of[i ^ 1];
                if (blk_pos[k] == M) return fail(SSS_EINVAL, "rotating pair split by the pruning");
            } else {
                bs[k] = p->slast[i - 2 * p->D];
            }
        }
        dbl.insert(dbl.end(), bs.begin(), bs.end());
        dbl.insert(dbl.end(), bp.begin(), bp.end());
    }
    ints.insert(ints.end(), row_orig.begin(), row_orig.end());
    const size_t o_bpos = ints.size();
    ints.insert(ints.end(), blk_pos.begin(), blk_pos.end());
    const size_t o_rbeg = ints.size();
    {
        int k = 0;
        ints.push_back(0);
        for (int l = 0; l < L; l++) {
            k += (int)Ly.lane_of[l].size();
            ints.push_back(k);
        }
    }
    size_t bytes = sizeof(double) * dbl.size() + sizeof(unsigned) * words.size() + sizeof(int) * ints.size();
    if (int rc = tables.ensure(bytes + 64)) return rc;
    std::vector<char> blob(bytes);
    memcpy(blob.data(), dbl.data(), sizeof(double) * dbl.size());
    memcpy(blob.data() + sizeof(double) * dbl.size(), words.data(), sizeof(unsigned) * words.size());
    memcpy(blob.data() + sizeof(double) * dbl.size() + sizeof(unsigned) * words.size(), ints.data(),
           sizeof(int) * ints.size());
    SSS_CUDA(cudaMemcpyAsync(tables.p, blob.data(), bytes, cudaMemcpyHostToDevice, st));
    if (int rc = p->w_queue.ensure(sizeof(int) * 4)) return rc;
    SSS_CUDA(cudaMemsetAsync(p->w_queue.p, 0, sizeof(int) * 4, st));
    const double* dv = tables.as<double>();
    const unsigned* dw = reinterpret_cast<const unsigned*>(dv + dbl.size());
    const int* di = reinterpret_cast<const int*>(dw + words.size());

    BatchArgs a{};
    a.M = M; a.Ga = Ga; a.K = p->d.K; a.Q = p->d.Q; a.F = F; a.nch = nch; a.nseg = nseg;
    a.T_max = 0; a.ntraj = ntraj; a.degree = degree; a.substeps = substeps; a.N = N;
    a.E = E;
    a.h_sub = dt / F / substeps; a.t0 = 0.0; a.dt = dt;
    for (int gi = 0; gi < Ga; gi++) a.gen_index[gi] = active[gi];
    a.W = p->d_gens.as<double>() + p->gens.size();
    a.gv = dv;
    a.rw = h_rw ? dv + n_gv : nullptr;
    a.toff = dv + n_gv + M;
    a.noff = a.toff + F;
    a.ent = dw;
    a.lane_rows = di;
    a.row_orig = di + n_lane_ints;
    a.rbeg = di + o_rbeg;
    if (Ly.parts) {
        a.pcol = di;
        a.cw = dw;
        a.om0 = dv + o_om0;
        a.kc = Ly.kc;
        a.n_live = (int)live.size();
        for (size_t i = 0; i < live.size(); i++) {
            a.live[i] = live[i];
            a.live_k[i] = live_k[i];
            a.live_ch[i] = live_ch[i];
        }
        a.n_lch = (int)lch.size();
        for (size_t i = 0; i < lch.size(); i++) a.lch_chan[i] = lch[i];
    }
    // pattern entries with a non-zero value in some live generator
    {
        int lnnz = 0;
        for (const auto& re : Ly.row_ents)
            for (const BatchLayout::Ent& en : re) {
                bool nz = false;
                for (int gi : live) nz |= p->sparse.val[(size_t)active[gi] * p->sparse.nnz + en.q] != 0.0;
                lnnz += nz;
            }
        p->mk_n_live = (int)live.size();
        p->mk_live_nnz = lnnz;
    }
    if (Ly.slots) {
        a.S = Ly.S;
        a.bar_at = Ly.bar_at;
        a.npart = Ly.npart;
        // per live generator, the slots where some lane holds a non-zero value
        for (size_t i = 0; i < live.size(); i++) {
            unsigned m = 0;
            for (int q = 0; q < Ly.S; q++)
                for (int l = 0; l < L; l++)
                    if (Ly.gv[((size_t)live[i] * Ly.S + q) * L + l] != 0.0) m |= 1u << q;
            a.amask[i] = m;
        }
        // scaled Horner coefficients c_j = d!/(j-1)! = j (j+1) ... d, and 1/d!
        for (int j = 0; j <= kMaxTaylor; j++) a.cfac[j] = 0.0;
        for (int j = 1; j <= degree; j++) {
            double c = 1.0;
            for (int k = j; k <= degree; k++) c *= k;
            a.cfac[j] = c;
        }
        a.inv_dfact = 1.0 / a.cfac[1];
    }
    a.rot = rot ? 1 : 0;
    a.resid = (p->d.flags & SSS_RESIDUAL) ? 1 : 0;
    if (rot) {
        a.Vm = p->d_V.as<double>();
        a.Vinvm = p->d_Vinv.as<double>();
        a.blk_self = dv + o_blk;
        a.blk_part = dv + o_blk + M;
        a.blk_pos = di + o_bpos;
    }
    a.rho0 = nullptr; a.prog = nullptr; a.samples = nullptr;
    a.tab = nullptr;
    a.tab_G = p->d.G;
    a.readout = nullptr; a.fin = nullptr;
    a.queue = p->w_queue.as<int>();
    for (int j = 0; j <= kMaxTaylor; j++) a.inv_j[j] = j ? 1.0 / j : 0.0;

    *out = a;
    if (Ly.slots) {
        const size_t per_slot = (3 * (size_t)(M + 2 + Ly.npart) +
                                 (size_t)kRing * (p->d.Q * lch.size() + p->d.K * live.size())) | 1;
        *smem = sizeof(double) * ((threads / L) * per_slot + M);
    } else if (Ly.parts) {
        const size_t per_slot = (3 * (size_t)(M + 2) + L * Ly.C + 1 +
                                 (size_t)kRing * (p->d.Q * lch.size() + p->d.K * live.size())) | 1;
        *smem = sizeof(double) * ((threads / L) * per_slot + M);
    } else if (use_reg) {
        const size_t per_slot = ((one_chain ? 4 : 5) * (size_t)M + kMaxQ * kMaxG) | 1;
        *smem = sizeof(double) * ((threads / L) * per_slot + M);
    } else {
        const size_t shared_words = (size_t)Ga * E * L + M + ((size_t)E * L + L + 1) / 2;
        const size_t per_slot = ((size_t)E * L + 3 * M + kMaxQ * kMaxG) | 1;
        *smem = sizeof(double) * (shared_words + (threads / L) * per_slot);
    }
    if (*smem > 227 * 1024)
        return fail(SSS_EINVAL, "batched kernel needs " + std::to_string(*smem) +
                                    " bytes of shared memory per CTA (max 232448); use fewer "
                                    "threads per CTA");
    return SSS_OK;
}

// trajectories of a prepared batch with more than t output samples
static int running_after(const sss_plan* p, int t) { return running_after(p->batch_longest, t); }

int batch_prepare(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg,
                  const double* d_prog, double dt, int F, const double* h_rw, cudaStream_t st,
                  const double* d_tab, int T_tab, const int* h_samples) {
    p->batch_ready = false;
    p->batch_empty = false;
    p->batch_nphases = 0;
    p->batch_longest.clear();
    p->batch_order = nullptr;
    if (d_tab) {
        nch = p->d.G;
        nseg = 0;
    }
    p->batch_table = d_tab != nullptr;
    p->batch_ntraj = ntraj;
    p->batch_nch = nch;
    p->batch_nseg = nseg;
    p->batch_dt = dt;
    p->batch_F = F;
    p->batch_has_rw = h_rw != nullptr;
    // uneven lengths: hand trajectories out longest first, so that the
    // groups sharing a warp run for about as long, the queue balances the
    // tail, and the trajectories still running are always the first ones
    // in the queue (longest-processing-time order)
    if (h_samples && ntraj > 1) {
        std::vector<int> order(ntraj);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(),
                         [&](int x, int y) { return h_samples[x] > h_samples[y]; });
        bool identity = true;
        for (int i = 0; i < ntraj && identity; i++) identity = order[i] == i;
        if (!identity) {
            if (int rc = p->w_order.ensure(sizeof(int) * (size_t)ntraj)) return rc;
            SSS_CUDA(cudaMemcpyAsync(p->w_order.p, order.data(), sizeof(int) * (size_t)ntraj,
                                     cudaMemcpyHostToDevice, st));
            SSS_CUDA(cudaStreamSynchronize(st));  // the host order goes out of scope
            p->batch_order = p->w_order.as<int>();
        }
    }
    // Phases.  The automatic lane count is the narrowest group that still
    // gives every SM sub-partition a warp (n * L >= 4*32*SMs lanes).  With
    // uneven lengths fewer groups remain as trajectories finish, whole
    // sub-partitions idle and the longest trajectories run at the speed of
    // one narrow group; so the batch is also laid out for the lane counts
    // the trajectories still running call for, each from the output sample
    // where the previous count stops meeting the rule (wider groups,
    // shorter chains per trajectory).  A launch switches layout at those
    // samples, as a chunked run switches chunks.
    const bool phased = h_samples && ntraj > 1 && p->batch_lanes == 0 &&
                        (p->batch_variant == 0 || p->batch_variant == 4 || p->batch_variant == 5 ||
                         p->batch_variant == 6 || p->batch_variant == 7);
    if (phased) {
        p->batch_longest.assign(h_samples, h_samples + ntraj);
        std::sort(p->batch_longest.begin(), p->batch_longest.end(), std::greater<int>());
    }
    int t = 0;
    for (int k = 0; k < kMaxPhases; k++) {
        BatchLayout Ly;
        p->auto_lanes_ntraj = phased ? std::max(1, running_after(p, t)) : 0;
        int rc = build_layout(p, ntraj, d_rho0, nch, nseg, d_prog, dt, F, {}, true, &Ly, st, false,
                              d_tab, T_tab);
        p->auto_lanes_ntraj = 0;
        if (rc) return rc;
        if (Ly.M == 0) {  // nothing reachable: the states stay as they are
            p->batch_empty = true;
            break;
        }
        if (k > 0 && Ly.L <= p->batch_phase[k - 1].L) break;  // no wider layout: phase k-1 runs on
        BatchArgs a{};
        size_t smem = 0;
        if (int rc2 = make_args(p, Ly, ntraj, nch, nseg, dt, F, h_rw, {}, p->batch_tables[k], &a,
                                &smem, st))
            return rc2;
        sss_plan::BatchPhase& ph = p->batch_phase[k];
        static_assert(sizeof(BatchArgs) <= sizeof(ph.args), "BatchArgs does not fit the plan");
        memcpy(ph.args, &a, sizeof(BatchArgs));
        ph.smem = smem;
        ph.L = Ly.L;
        ph.C = Ly.C;
        ph.P = Ly.P;
        ph.epl = Ly.epl;
        ph.threads = Ly.threads;
        ph.t_start = t;
        ph.use_reg = Ly.use_reg;
        ph.one_chain = p->batch_variant == 3;
        ph.parts = Ly.parts;
        ph.slots = Ly.slots;
        ph.phased = Ly.phased;
        ph.S = Ly.S;
        ph.shape = Ly.shape;
        // the register-state form: one trajectory per warp, one chain per
        // lane, no lane owning two rows, and a lane whose parts are all
        // padding (the zero partial of the padding close slots); lab frame
        ph.shfl = false;
        if (p->batch_variant == 5 && Ly.parts && !Ly.slots && Ly.L == 32 && Ly.C == 1 && !p->rotating) {
            bool ok = true, pad_lane = false;
            for (int l = 0; l < Ly.L && ok; l++) ok = Ly.lane_of[l].size() <= 1;
            for (int l = 0; l < Ly.L && !pad_lane; l++) {
                bool all = true;
                for (int q = 0; q < Ly.P; q++) all = all && Ly.pcol[(size_t)q * Ly.L + l] == Ly.M;
                pad_lane = all;
            }
            ph.shfl = ok && pad_lane && (Ly.P == 4 || Ly.P == 8);
        }
        p->batch_nphases = k + 1;
        if (k == 0) {
            p->last_batch_lanes = Ly.L;
            p->last_degree = Ly.degree;
            p->last_substeps = Ly.substeps;
            p->last_rows = Ly.M;
            p->last_nnz = (int)Ly.nnz;
            p->last_epl = Ly.E;
            p->last_active = Ly.Ga;
            p->last_variant = Ly.phased ? 7 : Ly.slots ? 6 : Ly.parts ? 4 : Ly.use_reg ? (ph.one_chain ? 3 : 1) : 2;
            p->last_n_live = p->mk_n_live;
            p->last_live_nnz = p->mk_live_nnz;
            p->last_fp64_per_term = Ly.slots ? Ly.S : Ly.parts ? Ly.C * Ly.P + Ly.kc : Ly.E;
        }
        if (!phased || !Ly.parts) break;
        // the next phase starts at the first sample where the automatic
        // lane count for the trajectories still running exceeds this one
        // (phases only widen; where the count drops back to a narrower group
        // on a tie the phase runs on)
        const int n_next = phase_end_count(4L * p->num_sms, p->auto_cost, Ly.L, running_after(p, t));
        if (n_next < 0 || p->batch_longest[n_next] <= t) break;
        t = p->batch_longest[n_next];
    }
    // the health word: all ones while every written value is finite
    if (int rc = p->w_health.ensure(sizeof(unsigned long long))) return rc;
    SSS_CUDA(cudaMemsetAsync(p->w_health.p, 0xff, sizeof(unsigned long long), st));
    p->batch_ready = true;
    return SSS_OK;
}

int batch_check(sss_plan* p, cudaStream_t st) {
    if (!p->w_health.p) return SSS_OK;
    unsigned long long h = ~0ull;
    SSS_CUDA(cudaMemcpyAsync(&h, p->w_health.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    SSS_CUDA(cudaStreamSynchronize(st));
    if (h == ~0ull) return SSS_OK;
    SSS_CUDA(cudaMemsetAsync(p->w_health.p, 0xff, sizeof(h), st));
    SSS_CUDA(cudaStreamSynchronize(st));
    return fail(SSS_ENONFINITE, "a state became NaN or Inf: trajectory " +
                                    std::to_string((unsigned)(h & 0xffffffffu)) +
                                    ", first at output sample " + std::to_string((unsigned)(h >> 32)));
}

int batch_launch(sss_plan* p, double* d_state, const double* d_prog, const int* d_samples,
                 double t0, int t_begin, int n_samples, int T_max, double* d_readout,
                 cudaStream_t st, double* d_trace, const double* d_tab) {
    if (!p->batch_ready) return fail(SSS_EINVAL, "no prepared batch (call sss_batch_prepare)");
    if (p->batch_table != (d_tab != nullptr))
        return fail(SSS_EINVAL, p->batch_table ? "the prepared batch runs from a coefficient table"
                                               : "the prepared batch runs from programs");
    p->last_launches = 0;
    if (p->batch_empty || n_samples <= 0) {
        if (d_readout && n_samples > 0)
            SSS_CUDA(cudaMemset2DAsync(d_readout + t_begin, sizeof(double) * T_max, 0,
                                       sizeof(double) * n_samples, p->batch_ntraj, st));
        return SSS_OK;
    }
    // The samples [t_begin, t_end) run as one launch per phase they touch,
    // and a phase's launch is cut again where the number of trajectories
    // still running halves (while at least two per SM remain): every launch
    // has one group per running trajectory, which the queue hands the
    // running ones first, so its CTAs spread evenly over the SMs.
    const int t_end = t_begin + n_samples;
    int launches = 0, rc = SSS_OK;
    for (int t = t_begin; t < t_end && rc == SSS_OK;) {
        int k = 0;
        while (k + 1 < p->batch_nphases && p->batch_phase[k + 1].t_start <= t) k++;
        int stop = t_end;
        if (k + 1 < p->batch_nphases) stop = std::min(stop, p->batch_phase[k + 1].t_start);
        int n_running = 0;
        if (!p->batch_longest.empty()) {
            n_running = running_after(p, t);
            if (n_running >= 4 * p->num_sms) {
                const int half_at = p->batch_longest[n_running / 2 - 1];
                if (half_at > t) stop = std::min(stop, half_at);
            }
        }
        const sss_plan::BatchPhase& ph = p->batch_phase[k];
        BatchArgs a;
        memcpy(&a, ph.args, sizeof(BatchArgs));
        a.rho0 = d_state;
        a.fin = d_state;
        a.prog = d_prog;
        a.samples = d_samples;
        a.readout = d_readout;
        a.trace = d_trace;
        a.order = p->batch_order;
        a.tab = d_tab;
        a.rw = d_readout ? a.rw : nullptr;
        a.health = p->w_health.as<unsigned long long>();
        a.t0 = t0;
        a.t_begin = t;
        a.t_end = stop;
        a.T_max = T_max;
        SSS_CUDA(cudaMemsetAsync(a.queue, 0, sizeof(int), st));
        const int L = ph.L, epl = ph.epl, threads = ph.threads;
        const size_t smem = ph.smem;
        p->ev_keep_begin = launches > 0;
        p->launch_active = n_running;
        if (ph.shfl) {
            rc = ph.P == 4 ? launch(p, k_batch_shfl<4>, a, threads, threads / 32, smem, st)
                           : launch(p, k_batch_shfl<8>, a, threads, threads / 32, smem, st);
        } else if (ph.phased) {
            rc = launch_phased(p, L, ph.shape, a, threads, smem, st);
        } else if (ph.slots) {
            rc = launch_slots(p, L, ph.S, a, threads, smem, st);
        } else if (ph.parts) {
            switch (L) {
                case 8: rc = launch_parts<8>(p, ph.C, ph.P, a, threads, smem, st); break;
                case 16: rc = launch_parts<16>(p, ph.C, ph.P, a, threads, smem, st); break;
                case 32: rc = launch_parts<32>(p, ph.C, ph.P, a, threads, smem, st); break;
                case 64: rc = launch_parts<64>(p, ph.C, ph.P, a, threads, smem, st); break;
                case 128: rc = launch_parts<128>(p, ph.C, ph.P, a, threads, smem, st); break;
                default: rc = launch_parts<256>(p, ph.C, ph.P, a, threads, smem, st); break;
            }
        } else if (ph.use_reg) {
            switch (L) {
                case 1: rc = launch_reg<1>(p, epl, a, threads, smem, st, ph.one_chain); break;
                case 2: rc = launch_reg<2>(p, epl, a, threads, smem, st, ph.one_chain); break;
                case 4: rc = launch_reg<4>(p, epl, a, threads, smem, st, ph.one_chain); break;
                case 8: rc = launch_reg<8>(p, epl, a, threads, smem, st, ph.one_chain); break;
                case 16: rc = launch_reg<16>(p, epl, a, threads, smem, st, ph.one_chain); break;
                default: rc = launch_reg<32>(p, epl, a, threads, smem, st, ph.one_chain); break;
            }
        } else {
            switch (L) {
                case 1: rc = launch(p, k_batch_lanes<1>, a, threads, threads, smem, st); break;
                case 2: rc = launch(p, k_batch_lanes<2>, a, threads, threads / 2, smem, st); break;
                case 4: rc = launch(p, k_batch_lanes<4>, a, threads, threads / 4, smem, st); break;
                case 8: rc = launch(p, k_batch_lanes<8>, a, threads, threads / 8, smem, st); break;
                case 16: rc = launch(p, k_batch_lanes<16>, a, threads, threads / 16, smem, st); break;
                default: rc = launch(p, k_batch_lanes<32>, a, threads, threads / 32, smem, st); break;
            }
        }
        p->ev_keep_begin = false;
        p->launch_active = 0;
        if (rc == SSS_OK) launches++;
        t = stop;
    }
    p->last_launches = launches;
    return rc;
}

int parts_forward_prepare(sss_plan* p, const BatchLayout& Ly, int ntraj, int nch, int nseg,
                          double dt, int F, const double* h_rw, const std::vector<int>& keep_live,
                          DevBuf& tables, PartsForward* fw, cudaStream_t st) {
    if (!Ly.parts) return fail(SSS_EINVAL, "not a row-part layout");
    BatchArgs a{};
    size_t smem = 0;
    if (int rc = make_args(p, Ly, ntraj, nch, nseg, dt, F, h_rw, keep_live, tables, &a, &smem, st))
        return rc;
    static_assert(sizeof(BatchArgs) <= sizeof(fw->args), "BatchArgs does not fit");
    memcpy(fw->args, &a, sizeof(BatchArgs));
    fw->smem = smem;
    fw->L = Ly.L;
    fw->C = Ly.C;
    fw->P = Ly.P;
    fw->threads = Ly.threads;
    return SSS_OK;
}

int parts_forward_launch(sss_plan* p, const PartsForward& fw, int ntraj, double* d_state,
                         const double* d_prog, double t0, int T, double* d_readout,
                         double* d_states, cudaStream_t st) {
    BatchArgs a;
    memcpy(&a, fw.args, sizeof(BatchArgs));
    a.ntraj = ntraj;
    a.rho0 = d_state;
    a.fin = d_state;
    a.prog = d_prog;
    a.samples = nullptr;
    a.readout = d_readout;
    a.rw = d_readout ? a.rw : nullptr;
    a.trace = nullptr;
    a.t0 = t0;
    a.t_begin = 0;
    a.t_end = T;
    a.T_max = T;
    a.states = d_states;
    a.st_steps = (long)T * a.F;
    SSS_CUDA(cudaMemsetAsync(a.queue, 0, sizeof(int), st));
    switch (fw.L) {
        case 8: return launch_parts<8>(p, fw.C, fw.P, a, fw.threads, fw.smem, st);
        case 16: return launch_parts<16>(p, fw.C, fw.P, a, fw.threads, fw.smem, st);
        case 32: return launch_parts<32>(p, fw.C, fw.P, a, fw.threads, fw.smem, st);
        case 64: return launch_parts<64>(p, fw.C, fw.P, a, fw.threads, fw.smem, st);
        case 128: return launch_parts<128>(p, fw.C, fw.P, a, fw.threads, fw.smem, st);
        default: return launch_parts<256>(p, fw.C, fw.P, a, fw.threads, fw.smem, st);
    }
}

int slot_layout_host(int M, const int* row_ptr, const int* col, int L, int S_cap, int* S_out,
                     int* bar_out, int* npart_out, unsigned* words, int* entries) {
    if (M < 0 || M + 2 > (int)kSlotIdx || !row_ptr || !S_out || !bar_out || !npart_out || !words ||
        !entries)
        return fail(SSS_EINVAL, "bad slot layout arguments");
    if (L != 8 && L != 16 && L != 32 && L != 64 && L != 128 && L != 256)
        return fail(SSS_EINVAL, "lanes must be 8, 16, 32, 64, 128 or 256");
    std::vector<int> nent(M);
    for (int i = 0; i < M; i++) {
        nent[i] = row_ptr[i + 1] - row_ptr[i];
        if (nent[i] < 0) return fail(SSS_EINVAL, "row_ptr must not decrease");
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++)
            if (!col || col[k] < 0 || col[k] >= M) return fail(SSS_EINVAL, "column out of range");
    }
    std::vector<SlotCell> cell;
    int S = 0, SA = 0, np = 0;
    if (!slots_pack(nent, L, std::min(S_cap, kSlotsMax), cell, &S, &SA, &np))
        return fail(SSS_EINVAL, "no slot layout up to the given number of slots");
    for (int q = 0; q < kSlotsMax; q++)
        for (int l = 0; l < L; l++) {
            const size_t o = (size_t)q * L + l;
            words[o] = (unsigned)M | kSlotStart;
            entries[o] = -1;
            if (q >= S) continue;
            const SlotCell& c = cell[(size_t)l * S + q];
            unsigned w = c.flags | ((unsigned)c.pidx << kSlotPidxShift);
            if (c.kind == 1) {
                w |= (unsigned)col[row_ptr[c.row] + c.ent];
                entries[o] = row_ptr[c.row] + c.ent;
            } else if (c.kind == 2) {
                w |= kSlotPart | (unsigned)c.part;
                entries[o] = -2;
            } else if (c.kind == 3) {
                w |= kSlotClose | (unsigned)c.row;
            } else {
                w = (unsigned)M | kSlotStart;
            }
            words[o] = w;
        }
    *S_out = S;
    *bar_out = SA;
    *npart_out = np;
    return SSS_OK;
}

int batch_run(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg, const double* d_prog,
              const int* d_samples, const int* h_samples, double t0, double dt, int T_max, int F,
              const double* h_rw, double* d_readout, double* d_final, cudaStream_t st,
              double* d_trace, const double* d_tab) {
    const int N = p->d.N;
    if (d_trace)
        SSS_CUDA(cudaMemsetAsync(d_trace, 0, sizeof(double) * (size_t)ntraj * T_max * N, st));
    if (int rc = batch_prepare(p, ntraj, d_rho0, nch, nseg, d_prog, dt, F, h_rw, st, d_tab, T_max,
                               h_samples))
        return rc;
    // the launches run in place on a state buffer that starts as rho0
    double* state = d_final;
    if (!state) {
        if (int rc = p->w_state.ensure(sizeof(double) * (size_t)ntraj * N)) return rc;
        state = p->w_state.as<double>();
    }
    if (state != d_rho0)
        SSS_CUDA(cudaMemcpyAsync(state, d_rho0, sizeof(double) * (size_t)ntraj * N,
                                 cudaMemcpyDeviceToDevice, st));
    return batch_launch(p, state, d_prog, d_samples, t0, 0, T_max, T_max, d_readout, st, d_trace,
                        d_tab);
}

}  // namespace sss
