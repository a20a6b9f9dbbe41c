// Adjoint gradients of a time-integrated readout with respect to the
// amplitudes and phases of the x-drive segments.  No reference
// counterpart: the reference has no derivatives.  The forward model is the
// reference's integrator exactly as the batched kernel runs it
// (superspinsim/generate_simulator.py:1954-2015 step structure, CF weights
// :278-350, exponential K-1 first :1259-1294).
//
// Objective (per trajectory):  J = sum_t tw[t] * rw . rho(t0 + dt*(t+1)).
// Parameters: for every segment s of channel 0 (the x field), its amplitude
// a_s and phase phi_s (c_x(t) = offset + a_s cos(tau f t + phi_s)).
//
// Every parameter enters a step's exponent Omega_e only through the scalar
// coefficient of Gx, so dOmega_e/dtheta = beta_e(theta) Gx with
// beta_e = h sum_k W[e,k] dc_x(t_k)/dtheta, and
//     dJ/dtheta = sum_steps sum_e beta_e * g_e,
//     g_e = mu_after^T L(Omega_e, Gx) rho_before,
// L the Frechet derivative of exp.  With the exponential truncated at
// degree d (as the forward pass evaluates it), L(Omega, G) is exactly
// sum_{a+b<=d-1} Omega^a G Omega^b / (a+b+1)!, so
//     g_e = sum_{a+b<=d-1} (u_a . z_b) / (a+b+1)!,
//     u_a = (Omega^T)^a mu,  z_b = G Omega^b rho,
// and the adjoint itself moves as mu <- sum_{a<=d} u_a / a!  (= E^T mu).
// Both come from one series: g_e = rho^T L(Omega^T, G^T) mu, and the
// block matrix [[Omega^T, G^T], [0, Omega^T]] applied to [0; mu] by Horner
// (degree d) gives L(Omega^T, G^T) mu on top and E^T mu below -- per term
// two transposed products with Omega and one with G, no dot products.
//
// Checkpointing: the forward pass keeps the state every C ~ sqrt(steps)
// steps; the backward sweep recomputes one interval at a time (storing the
// state before each exponential) and walks it in reverse.  Memory per
// trajectory in flight: (steps/C + C*K) * rows doubles.
//
// Layout and parallel structure are the batched kernel's shared-memory
// variant: a group of L lanes per trajectory, rows split across lanes,
// a device work queue.  The transposed products use a second per-lane entry
// list that points into the same assembled Omega.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "sss_device.cuh"
#include "sss_internal.cuh"

namespace sss {
namespace {

constexpr int kAdjMaxTaylor = 24;

struct AdjArgs {
    int M, Ga, K, Q, F, nch, nseg, ntraj, degree, N, E, ET;
    int xg;          // position of Gx among the active generators
    long n_steps;    // fine steps per trajectory
    int T, C, n_ck;
    double h, t0, dt;
    int gen_index[kMaxG];
    const double* toff;
    const double* noff;
    const double* W;
    const double* gv;       // Ga*E*L
    const unsigned* ent;    // E*L
    const int* cnt;         // L
    const int* rbeg;        // L+1 first row of each lane (lane order)
    const unsigned* tent;   // ET*L transposed words
    const int* tidx;        // ET*L index into Om (e*L + l), -1: zero
    const int* tcnt;        // L
    const int* row_orig;    // M
    const double* rw;       // M (compressed)
    const double* tw;       // T
    const double* rho0;     // ntraj*N
    const double* prog;     // ntraj*nch*nseg*5
    double* J;              // ntraj
    double* grad;           // ntraj*nseg*2
    double* ck;             // slots*n_ck*M
    double* st;             // slots*C*K*M
    int* queue;
    double fact_inv[kAdjMaxTaylor + 2];
    double inv_j[kAdjMaxTaylor + 1];
};

__device__ __forceinline__ int wcol(unsigned w) { return (int)(w & 0xffffu); }
__device__ __forceinline__ int wend(unsigned w) { return (int)(w >> 16); }
// transposed-entry index flag: the x generator is non-zero at this entry
constexpr int kHasG = 1 << 30;

// x-channel segment at time t: index (or -1) and its parameters
__device__ __forceinline__ int x_segment(const double* prog, int nseg, double t) {
    for (int s = 0; s < nseg; s++)
        if (t < prog[s * 5]) return s;
    return -1;
}

template <int L>
struct Group {
    int li;
    unsigned gmask;
    unsigned leader;
    int nE, nET, r0, r1;
    const unsigned* s_ent;
    const unsigned* s_tent;
    const int* s_tidx;
    __device__ void sync() const { __syncwarp(gmask); }
    __device__ double sum(double x) const {
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) x += __shfl_xor_sync(gmask, x, o);
        return x;
    }
    // out[row] = sum Om[e] in[col] over this lane's rows; optional Horner
    // form out = base + (.)*scale
    __device__ void fwd(const double* Om, const double* in, double* out, const double* base,
                        double scale) const {
        double s = 0.0;
        for (int e = 0; e < nE; e++) {
            unsigned w = s_ent[e * L + li];
            s = fma(Om[e * L + li], in[wcol(w)], s);
            if (wend(w)) {
                int row = wend(w) - 1;
                out[row] = base ? fma(s, scale, base[row]) : s;
                s = 0.0;
            }
        }
    }
    __device__ void trans(const double* Om, const double* in, double* out) const {
        double s = 0.0;
        for (int e = 0; e < nET; e++) {
            unsigned w = s_tent[e * L + li];
            int q = s_tidx[e * L + li];
            if (q >= 0) s = fma(Om[q & ~kHasG], in[wcol(w)], s);
            if (wend(w)) {
                out[wend(w) - 1] = s;
                s = 0.0;
            }
        }
    }
    // px_out = (Om^T px + G^T py)*scale, py_out = base + (Om^T py)*scale on
    // this lane's rows (G^T values read through the same entry indices)
    __device__ void trans_block(const double* Om, const double* Gv, const double* px,
                                const double* py, double* px_out, double* py_out,
                                const double* base, double scale) const {
        double s1 = 0.0, s2 = 0.0;
        for (int e = 0; e < nET; e++) {
            unsigned w = s_tent[e * L + li];
            int q = s_tidx[e * L + li];
            if (q >= 0) {
                const int c = wcol(w);
                const bool has_g = (q & kHasG) != 0;
                q &= ~kHasG;
                const double o = Om[q], pyc = py[c];
                s1 = fma(o, px[c], s1);
                if (has_g) s1 = fma(Gv[q], pyc, s1);
                s2 = fma(o, pyc, s2);
            }
            if (wend(w)) {
                const int row = wend(w) - 1;
                px_out[row] = s1 * scale;
                py_out[row] = fma(s2, scale, base[row]);
                s1 = 0.0;
                s2 = 0.0;
            }
        }
    }
    __device__ double dot(const double* a, const double* b) const {
        double s = 0.0;
        for (int i = r0; i < r1; i++) s = fma(a[i], b[i], s);
        return s;
    }
};

template <int L>
__global__ void __launch_bounds__(256) k_adjoint(const AdjArgs a) {
    extern __shared__ double smem[];
    const int M = a.M, Ga = a.Ga, E = a.E, ET = a.ET, d = a.degree, Q = a.Q, K = a.K;
    double* s_gv = smem;                                   // Ga*E*L
    double* s_rw = s_gv + (size_t)Ga * E * L;              // M
    unsigned* s_ent = reinterpret_cast<unsigned*>(s_rw + M);
    unsigned* s_tent = s_ent + (size_t)E * L;
    int* s_tidx = reinterpret_cast<int*>(s_tent + (size_t)ET * L);
    const size_t shared_words = (size_t)Ga * E * L + M + ((size_t)E * L + 2 * (size_t)ET * L + 1) / 2;
    const size_t per_slot = ((size_t)E * L + 7 * (size_t)M + kMaxQ * kMaxG + 4 * kMaxQ) | 1;
    const int slot = threadIdx.x / L, li = threadIdx.x % L;
    double* Om = smem + shared_words + slot * per_slot;
    double* v = Om + (size_t)E * L;      // state
    double* bA = v + M;                  // Horner / power buffers
    double* bB = bA + M;
    double* mu = bB + M;
    double* mun = mu + M;
    double* u0 = mun + M;
    double* u1 = u0 + M;
    double* coef = u1 + M;               // Q*Ga
    double* nd = coef + kMaxQ * kMaxG;   // per node: cos, -amp*sin, segment (as double), used

    for (int i = threadIdx.x; i < Ga * E * L; i += blockDim.x) s_gv[i] = a.gv[i];
    for (int i = threadIdx.x; i < M; i += blockDim.x) s_rw[i] = a.rw ? a.rw[i] : 0.0;
    for (int i = threadIdx.x; i < E * L; i += blockDim.x) s_ent[i] = a.ent[i];
    for (int i = threadIdx.x; i < ET * L; i += blockDim.x) {
        s_tent[i] = a.tent[i];
        s_tidx[i] = a.tidx[i];
    }
    __syncthreads();

    Group<L> grp;
    grp.li = li;
    const unsigned lane_in_warp = threadIdx.x & 31;
    grp.leader = lane_in_warp / L * L;
    grp.gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << grp.leader);
    grp.nE = __ldg(a.cnt + li);
    grp.nET = __ldg(a.tcnt + li);
    grp.r0 = __ldg(a.rbeg + li);
    grp.r1 = __ldg(a.rbeg + li + 1);
    grp.s_ent = s_ent;
    grp.s_tent = s_tent;
    grp.s_tidx = s_tidx;
    const long gslot = (long)blockIdx.x * (blockDim.x / L) + slot;
    double* ck = a.ck + gslot * (long)a.n_ck * M;
    double* st = a.st + gslot * (long)a.C * K * M;

    // coefficients of step n at the Q nodes; with derivs, also the x
    // channel's segment and its derivative factors at each node
    auto coefficients = [&](const double* prog, long n, bool derivs) {
        const int t = (int)(n / a.F), r = (int)(n % a.F);
        for (int i = li; i < Q * Ga; i += L) {
            int k = i / Ga, g = a.gen_index[i - k * Ga];
            double val = 1.0;
            if (g > 0) {
                double tn = __dadd_rn(__dadd_rn(__dadd_rn(a.t0, __ldg(a.toff + r)),
                                                __dmul_rn(a.dt, (double)t)),
                                      __ldg(a.noff + k));
                val = (g - 1 < a.nch) ? channel_value(prog, a.nseg, g - 1, tn) : 0.0;
            }
            coef[i] = val;
        }
        if (derivs && li < Q) {
            const int k = li;
            double tn = __dadd_rn(__dadd_rn(__dadd_rn(a.t0, __ldg(a.toff + r)),
                                            __dmul_rn(a.dt, (double)t)),
                                  __ldg(a.noff + k));
            int s = x_segment(prog, a.nseg, tn);
            double cs = 0.0, dph = 0.0;
            if (s >= 0) {
                const double* p = prog + s * 5;
                double arg = __dadd_rn(__dmul_rn(__dmul_rn(6.283185307179586, p[3]), tn), p[4]);
                double sn, cn;
                sincos(arg, &sn, &cn);
                cs = cn;
                dph = -p[2] * sn;
            }
            nd[4 * k] = cs;
            nd[4 * k + 1] = dph;
            nd[4 * k + 2] = (double)s;
        }
        grp.sync();
    };
    auto assemble = [&](int e) {
        double ag[kMaxG];
        for (int g = 0; g < Ga; g++) {
            double s = 0.0;
            for (int k = 0; k < Q; k++) s = fma(__ldg(a.W + e * Q + k), coef[k * Ga + g], s);
            ag[g] = s * a.h;
        }
        for (int q = 0; q < grp.nE; q++) {
            double o = 0.0;
            for (int g = 0; g < Ga; g++) o = fma(ag[g], s_gv[((size_t)g * E + q) * L + li], o);
            Om[q * L + li] = o;
        }
        grp.sync();
    };
    // v <- exp(Om) v, Horner
    auto expv = [&]() {
        const double* cur = v;
        double* nxt = bA;
        for (int j = d; j >= 1; j--) {
            grp.fwd(Om, cur, nxt, v, a.inv_j[j]);
            grp.sync();
            cur = nxt;
            nxt = (nxt == bA) ? bB : bA;
        }
        for (int i = grp.r0; i < grp.r1; i++) v[i] = cur[i];
        grp.sync();
    };

    while (true) {
        int nb = 0;
        if (li == 0) nb = atomicAdd(a.queue, 1);
        const int b = __shfl_sync(grp.gmask, nb, grp.leader);
        if (b >= a.ntraj) break;
        const double* prog = a.prog + (size_t)b * a.nch * a.nseg * 5;
        const double* xprog = prog;  // channel 0 = x
        // ---- forward with checkpoints ----
        for (int i = grp.r0; i < grp.r1; i++) v[i] = a.rho0[(size_t)b * a.N + a.row_orig[i]];
        grp.sync();
        double Jacc = 0.0;
        for (long n = 0; n < a.n_steps; n++) {
            if (n % a.C == 0) {
                double* c = ck + (n / a.C) * M;
                for (int i = grp.r0; i < grp.r1; i++) c[i] = v[i];
            }
            coefficients(prog, n, false);
            for (int e = K - 1; e >= 0; e--) {
                assemble(e);
                expv();
            }
            if ((n + 1) % a.F == 0) {
                int t = (int)((n + 1) / a.F) - 1;
                Jacc = fma(a.tw[t], grp.sum(grp.dot(s_rw, v)), Jacc);
            }
        }
        if (li == 0) a.J[b] = Jacc;
        double* gb = a.grad + (size_t)b * a.nseg * 2;
        if (li == 0)
            for (int s = 0; s < 2 * a.nseg; s++) gb[s] = 0.0;
        // ---- backward ----
        for (int i = grp.r0; i < grp.r1; i++) mu[i] = 0.0;
        grp.sync();
        for (long c = a.n_ck - 1; c >= 0; c--) {
            const long n0 = c * a.C, n1 = min(n0 + (long)a.C, a.n_steps);
            for (int i = grp.r0; i < grp.r1; i++) v[i] = ck[c * M + i];
            grp.sync();
            for (long n = n0; n < n1; n++) {
                coefficients(prog, n, false);
                for (int e = K - 1; e >= 0; e--) {
                    double* s = st + ((n - n0) * K + e) * M;
                    for (int i = grp.r0; i < grp.r1; i++) s[i] = v[i];
                    assemble(e);
                    expv();
                }
            }
            for (long n = n1 - 1; n >= n0; n--) {
                if ((n + 1) % a.F == 0) {
                    const double w = a.tw[(n + 1) / a.F - 1];
                    for (int i = grp.r0; i < grp.r1; i++) mu[i] = fma(w, s_rw[i], mu[i]);
                }
                coefficients(prog, n, true);
                for (int e = 0; e < K; e++) {
                    assemble(e);
                    const double* s = st + ((n - n0) * K + e) * M;
                    for (int i = grp.r0; i < grp.r1; i++) v[i] = s[i];
                    grp.sync();
                    // Transposed block series on [0; mu]:
                    //   px <- (Om^T px + G^T py)/j,  py <- mu + (Om^T py)/j,
                    // j = d..1; then py = E^T mu and px = L(Om^T, G^T) mu,
                    // so g = rho_before . px.
                    double* pxc = mun;   // zero on entry
                    double* pyc = mu;
                    double* pxn = u0;
                    double* pyn = u1;
                    for (int i = grp.r0; i < grp.r1; i++) mun[i] = 0.0;
                    grp.sync();
                    for (int j = d; j >= 1; j--) {
                        grp.trans_block(Om, s_gv + (size_t)a.xg * E * L, pxc, pyc, pxn, pyn, mu,
                                        a.inv_j[j]);
                        grp.sync();
                        if (j == d) {
                            // pxc/pyc were mun/mu; move to the ping-pong pair
                            pxc = pxn; pyc = pyn;
                            pxn = bA; pyn = bB;
                        } else {
                            double* t1 = pxc; pxc = pxn; pxn = t1;
                            double* t2 = pyc; pyc = pyn; pyn = t2;
                        }
                    }
                    const double g = grp.sum(grp.dot(v, pxc));
                    for (int i = grp.r0; i < grp.r1; i++) mu[i] = pyc[i];
                    grp.sync();
                    if (li == 0) {
                        for (int k = 0; k < Q; k++) {
                            int sgm = (int)nd[4 * k + 2];
                            if (sgm < 0) continue;
                            double hw = a.h * __ldg(a.W + e * Q + k);
                            gb[2 * sgm] = fma(hw * nd[4 * k], g, gb[2 * sgm]);
                            gb[2 * sgm + 1] = fma(hw * nd[4 * k + 1], g, gb[2 * sgm + 1]);
                        }
                    }
                    grp.sync();
                }
            }
        }
        (void)xprog;
    }
}

template <int L>
int launch_adj(sss_plan* p, const AdjArgs& a, int threads, size_t smem, int grid, cudaStream_t st) {
    SSS_CUDA(cudaFuncSetAttribute(k_adjoint<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_adjoint<L><<<grid, threads, smem, st>>>(a);
    SSS_CUDA(cudaGetLastError());
    (void)p;
    return SSS_OK;
}

}  // namespace

int adjoint_run(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg,
                const double* d_prog, double t0, double dt, int T, int F, const double* h_rw,
                const double* h_tw, double* d_J, double* d_grad, cudaStream_t st) {
    const int N = p->d.N, K = p->d.K, Q = p->d.Q;
    if (p->d.G < 2) return fail(SSS_EINVAL, "the adjoint needs the x generator (G >= 2)");
    BatchLayout Ly;
    if (int rc = build_layout(p, ntraj, d_rho0, nch, nseg, d_prog, dt, F, {1}, false, &Ly, st))
        return rc;
    SSS_CUDA(cudaMemsetAsync(d_J, 0, sizeof(double) * ntraj, st));
    SSS_CUDA(cudaMemsetAsync(d_grad, 0, sizeof(double) * (size_t)ntraj * nseg * 2, st));
    if (Ly.M == 0) return SSS_OK;
    if (Ly.substeps != 1)
        return fail(SSS_EINVAL, "the adjoint needs one sub-step per exponential (use a smaller dt/F)");
    int xg = -1;
    for (int gi = 0; gi < Ly.Ga; gi++)
        if (Ly.active[gi] == 1) xg = gi;
    if (xg < 0) return fail(SSS_EINVAL, "the x generator is zero on the reachable rows");
    const int M = Ly.M, L = Ly.L, E = Ly.E, d = Ly.degree;
    if (d > kAdjMaxTaylor) return fail(SSS_EINVAL, "Taylor degree too large for the adjoint");
    // lane row ranges (lane order) and owner of each row
    std::vector<int> rbeg(L + 1, 0), owner(M, 0);
    for (int l = 0; l < L; l++) rbeg[l + 1] = rbeg[l] + (int)Ly.lane_of[l].size();
    for (int l = 0; l < L; l++)
        for (int k = rbeg[l]; k < rbeg[l + 1]; k++) owner[k] = l;
    // transposed entries: for each forward entry (row r, col c) at Om index
    // e*L + l, an entry (row c, col r) of the owner of c
    std::vector<std::vector<std::pair<int, std::pair<int, int>>>> trows(M);  // row c -> (col r, q)
    for (int l = 0; l < L; l++) {
        int e = 0;
        for (int i : Ly.lane_of[l]) {
            const auto& ents = Ly.row_ents[i];
            int n = std::max<int>(1, (int)ents.size());
            for (int j = 0; j < (int)ents.size(); j++) {
                int r = Ly.newpos[i], c = Ly.newpos[ents[j].col];
                trows[c].push_back({r, {e + j, l}});
            }
            e += n;
        }
    }
    std::vector<int> tcnt(L, 0);
    for (int l = 0; l < L; l++)
        for (int k = rbeg[l]; k < rbeg[l + 1]; k++) tcnt[l] += std::max<int>(1, (int)trows[k].size());
    const int ET = *std::max_element(tcnt.begin(), tcnt.end());
    std::vector<unsigned> tent((size_t)ET * L, 0u);
    std::vector<int> tidx((size_t)ET * L, -1);
    for (int l = 0; l < L; l++) {
        int e = 0;
        for (int k = rbeg[l]; k < rbeg[l + 1]; k++) {
            auto& lst = trows[k];
            std::sort(lst.begin(), lst.end());
            int n = std::max<int>(1, (int)lst.size());
            for (int j = 0; j < n; j++) {
                unsigned w = j < (int)lst.size() ? (unsigned)lst[j].first : (unsigned)k;
                if (j == n - 1) w |= (unsigned)(k + 1) << 16;
                tent[(size_t)(e + j) * L + l] = w;
                if (j < (int)lst.size()) {
                    const int fe = lst[j].second.first, fl = lst[j].second.second;
                    int q = fe * L + fl;
                    if (Ly.gv[((size_t)xg * E + fe) * L + fl] != 0.0) q |= kHasG;
                    tidx[(size_t)(e + j) * L + l] = q;
                }
            }
            e += n;
        }
    }
    const long n_steps = (long)T * F;
    int C = (int)std::ceil(std::sqrt((double)n_steps));
    C = std::max(C, 1);
    const int n_ck = (int)((n_steps + C - 1) / C);
    std::vector<double> rw(M, 0.0), tw(h_tw, h_tw + T);
    for (int k = 0; k < M; k++) rw[k] = h_rw ? h_rw[Ly.row_orig[k]] : 0.0;
    std::vector<double> toff(F), noff(Q);
    for (int r = 0; r < F; r++) toff[r] = ((double)r * dt) / F;
    for (int k = 0; k < Q; k++) noff[k] = (dt * p->nodes[k]) / F;
    // device blob: gv | rw | tw | toff | noff | ent | tent | tidx | cnt | tcnt | rbeg | row_orig
    std::vector<double> dbl(Ly.gv);
    const size_t o_rw = dbl.size();
    dbl.insert(dbl.end(), rw.begin(), rw.end());
    const size_t o_tw = dbl.size();
    dbl.insert(dbl.end(), tw.begin(), tw.end());
    const size_t o_toff = dbl.size();
    dbl.insert(dbl.end(), toff.begin(), toff.end());
    const size_t o_noff = dbl.size();
    dbl.insert(dbl.end(), noff.begin(), noff.end());
    std::vector<int> ints;
    auto put = [&](const int* b, size_t n) {
        size_t o = ints.size();
        ints.insert(ints.end(), b, b + n);
        return o;
    };
    const size_t o_ent = put(reinterpret_cast<const int*>(Ly.words.data()), Ly.words.size());
    const size_t o_tent = put(reinterpret_cast<const int*>(tent.data()), tent.size());
    const size_t o_tidx = put(tidx.data(), tidx.size());
    const size_t o_cnt = put(Ly.cnt.data(), Ly.cnt.size());
    const size_t o_tcnt = put(tcnt.data(), tcnt.size());
    const size_t o_rbeg = put(rbeg.data(), rbeg.size());
    const size_t o_rorig = put(Ly.row_orig.data(), Ly.row_orig.size());
    const size_t bytes = sizeof(double) * dbl.size() + sizeof(int) * ints.size();
    if (int rc = p->w_aux.ensure(bytes + 64)) return rc;
    std::vector<char> blob(bytes);
    memcpy(blob.data(), dbl.data(), sizeof(double) * dbl.size());
    memcpy(blob.data() + sizeof(double) * dbl.size(), ints.data(), sizeof(int) * ints.size());
    SSS_CUDA(cudaMemcpyAsync(p->w_aux.p, blob.data(), bytes, cudaMemcpyHostToDevice, st));
    const double* dv = p->w_aux.as<double>();
    const int* di = reinterpret_cast<const int*>(dv + dbl.size());

    const int threads = p->batch_threads > 0 ? p->batch_threads : 64;
    if (threads % L) return fail(SSS_EINVAL, "CTA size must be a multiple of the lanes per trajectory");
    const int slots_per_cta = threads / L;
    const size_t shared_words = (size_t)Ly.Ga * E * L + M + ((size_t)E * L + 2 * (size_t)ET * L + 1) / 2;
    const size_t per_slot = ((size_t)E * L + 7 * (size_t)M + kMaxQ * kMaxG + 4 * kMaxQ) | 1;
    const size_t smem = sizeof(double) * (shared_words + slots_per_cta * per_slot);
    if (smem > 227 * 1024) return fail(SSS_EINVAL, "adjoint kernel: shared memory per CTA too large");
    int grid = std::max(1, (ntraj + slots_per_cta - 1) / slots_per_cta);
    grid = std::min(grid, p->num_sms * 8);
    const long slots = (long)grid * slots_per_cta;
    const size_t scratch = sizeof(double) * (size_t)slots * ((size_t)n_ck * M + (size_t)C * K * M);
    if (int rc = p->w_prop.ensure(scratch)) return rc;
    if (int rc = p->w_queue.ensure(sizeof(int) * 4)) return rc;
    SSS_CUDA(cudaMemsetAsync(p->w_queue.p, 0, sizeof(int) * 4, st));

    AdjArgs a{};
    a.M = M; a.Ga = Ly.Ga; a.K = K; a.Q = Q; a.F = F; a.nch = nch; a.nseg = nseg;
    a.ntraj = ntraj; a.degree = d; a.N = N; a.E = E; a.ET = ET; a.xg = xg;
    a.n_steps = n_steps; a.T = T; a.C = C; a.n_ck = n_ck;
    a.h = dt / F; a.t0 = t0; a.dt = dt;
    for (int gi = 0; gi < Ly.Ga; gi++) a.gen_index[gi] = Ly.active[gi];
    a.toff = dv + o_toff;
    a.noff = dv + o_noff;
    a.W = p->d_gens.as<double>() + p->gens.size();
    a.gv = dv;
    a.rw = dv + o_rw;
    a.tw = dv + o_tw;
    a.ent = reinterpret_cast<const unsigned*>(di + o_ent);
    a.tent = reinterpret_cast<const unsigned*>(di + o_tent);
    a.tidx = di + o_tidx;
    a.cnt = di + o_cnt;
    a.tcnt = di + o_tcnt;
    a.rbeg = di + o_rbeg;
    a.row_orig = di + o_rorig;
    a.rho0 = d_rho0;
    a.prog = d_prog;
    a.J = d_J;
    a.grad = d_grad;
    a.ck = p->w_prop.as<double>();
    a.st = a.ck + (size_t)slots * n_ck * M;
    a.queue = p->w_queue.as<int>();
    double f = 1.0;
    for (int j = 0; j < kAdjMaxTaylor + 2; j++) {
        if (j > 0) f /= j;
        a.fact_inv[j] = f;
    }
    for (int j = 0; j <= kAdjMaxTaylor; j++) a.inv_j[j] = j ? 1.0 / j : 0.0;
    if (!p->ev_begin) {
        SSS_CUDA(cudaEventCreate(&p->ev_begin));
        SSS_CUDA(cudaEventCreate(&p->ev_end));
    }
    SSS_CUDA(cudaEventRecord(p->ev_begin, st));
    int rc;
    switch (L) {
        case 1: rc = launch_adj<1>(p, a, threads, smem, grid, st); break;
        case 2: rc = launch_adj<2>(p, a, threads, smem, grid, st); break;
        case 4: rc = launch_adj<4>(p, a, threads, smem, grid, st); break;
        case 8: rc = launch_adj<8>(p, a, threads, smem, grid, st); break;
        case 16: rc = launch_adj<16>(p, a, threads, smem, grid, st); break;
        default: rc = launch_adj<32>(p, a, threads, smem, grid, st); break;
    }
    if (rc) return rc;
    SSS_CUDA(cudaEventRecord(p->ev_end, st));
    p->ev_recorded = true;
    p->last_launches = 1;
    p->last_batch_lanes = L;
    p->last_degree = d;
    p->last_substeps = 1;
    p->last_rows = M;
    p->last_nnz = (int)Ly.nnz;
    return SSS_OK;
}

}  // namespace sss
