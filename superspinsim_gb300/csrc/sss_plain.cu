// Plain per-trajectory path: the drop-in for `simulate`
// (reference superspinsim/generate_simulator.py:1508-2200).
//
// The reference builds one step propagator per output sample, all samples
// in parallel (its only parallel axis), by F serial fine steps of K
// exponentials each, then chains them serially on the host with 2(T-1)
// launches and applies the cumulative propagators to rho0.  Here:
//
//  k_step_propagators: one CTA per (trajectory, output sample).  The N x N
//    working set (exponent, Taylor powers, exponential, accumulated step
//    propagator) lives in shared memory for the whole F x K fine-step loop;
//    generators stream from L2.  The exponential is either the reference's
//    own scheme (first-order Taylor after 4^-R scaling, 2R squarings; exact
//    operation order of :534-578, :706-724) or a degree-12 Taylor
//    polynomial (Paterson-Stockmeyer, 5 products) after norm-chosen
//    scaling, in residual form.
//  k_chain: one CTA per trajectory applies the T step propagators to the
//    state in order (v <- v + S_t v), an O(T N^2) serial tail instead of the
//    reference's O(T N^3) chain of matrix products, and writes the state
//    after every sample (mapped back from the rotating eigenbasis if used).
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "sss_device.cuh"
#include "sss_internal.cuh"

namespace sss {
namespace {

constexpr int kPlainThreads = 256;

// C = A*B + ca*A + cb*B  (C must alias neither A nor B)
__device__ void mm(double* __restrict__ C, const double* __restrict__ A,
                   const double* __restrict__ B, int N, double ca, double cb) {
    for (int idx = threadIdx.x; idx < N * N; idx += blockDim.x) {
        int i = idx / N, j = idx - i * N;
        double acc = ca * A[idx] + cb * B[idx];
        const double* a = A + i * N;
#pragma unroll 4
        for (int k = 0; k < N; k++) acc = fma(a[k], B[k * N + j], acc);
        C[idx] = acc;
    }
}

// Reference order products (generate_simulator.py:706-743): the running
// sum starts at (2*in) or (L + R) and adds the products k = 0..N-1.
__device__ void mm_ref(double* __restrict__ C, const double* __restrict__ A,
                       const double* __restrict__ B, int N, bool square,
                       bool residual) {
    for (int idx = threadIdx.x; idx < N * N; idx += blockDim.x) {
        int i = idx / N, j = idx - i * N;
        double acc = 0.0;
        if (residual) acc = square ? 2 * A[idx] : A[idx] + B[idx];
        for (int k = 0; k < N; k++) acc = fma(A[i * N + k], B[k * N + j], acc);
        C[idx] = acc;
    }
}

struct PlainArgs {
    int N, G, K, Q, F, T, nch, nseg, expm, R;
    int t_offset;  // global index of this launch's first output sample
    bool residual, rotating;
    const double* gens;   // G*N*N or Q*G*N*N
    const double* W;      // K*Q (device)
    const double* nodes;  // Q
    const double* dlast;  // D*2
    const double* slast;  // S
    int D, S;
    const double* prog;   // ntraj*nch*nseg*5
    const double* tab;    // ntraj*(F*T*Q)*G
    double t0, dt;
    double* out;          // ntraj*T*N*N
};

__global__ void __launch_bounds__(kPlainThreads)
k_step_propagators(PlainArgs a) {
    extern __shared__ double sm[];
    const int N = a.N, NN = N * N;
    const int t = blockIdx.x, b = blockIdx.y;
    double* X = sm;
    double* X2 = X + NN;
    double* X3 = X2 + NN;
    double* X4 = X3 + NN;
    double* Bm = X4 + NN;
    double* E = Bm + NN;
    double* TE = E + NN;
    double* T2 = TE + NN;
    __shared__ double coef[kMaxQ * kMaxG];
    __shared__ double colsum[64];
    const double h = a.dt / a.F;
    const double* prog = a.prog ? a.prog + (size_t)b * a.nch * a.nseg * 5 : nullptr;

    for (int i = threadIdx.x; i < NN; i += blockDim.x)
        TE[i] = (!a.residual && (i / N == i % N)) ? 1.0 : 0.0;

    for (int r = 0; r < a.F; r++) {
        __syncthreads();
        if (threadIdx.x < a.Q * a.G) {
            int k = threadIdx.x / a.G, g = threadIdx.x - k * a.G;
            double v;
            if (a.tab) {
                v = a.tab[(((size_t)b * a.F + r) * a.T + t) * a.Q * a.G + threadIdx.x];
            } else {
                double tn = node_time(a.t0, a.dt, a.F, r, a.t_offset + t, a.nodes[k]);
                if (!a.rotating)
                    v = (g == 0) ? 1.0 : (g - 1 < a.nch ? channel_value(prog, a.nseg, g - 1, tn) : 0.0);
                else
                    v = g < a.nch ? channel_value(prog, a.nseg, g, tn) : 0.0;
            }
            coef[k * a.G + g] = v;
        }
        __syncthreads();
        for (int e = a.K - 1; e >= 0; e--) {
            // exponent (generate_simulator.py:354-448 lab, :450-532 rotating)
            double wc[kMaxG];
            if (!a.rotating) {
                for (int g = 0; g < a.G; g++) {
                    double acc = 0.0;
                    for (int k = 0; k < a.Q; k++) acc = fma(a.W[e * a.Q + k], coef[k * a.G + g], acc);
                    wc[g] = acc;
                }
            }
            for (int idx = threadIdx.x; idx < NN; idx += blockDim.x) {
                double acc = 0.0;
                if (!a.rotating) {
                    for (int g = 0; g < a.G; g++) acc = fma(wc[g], __ldg(a.gens + (size_t)g * NN + idx), acc);
                    acc *= h;
                } else {
                    for (int k = 0; k < a.Q; k++) {
                        double m1 = h * a.W[e * a.Q + k];
                        for (int g = 0; g < a.G; g++)
                            acc = fma(__ldg(a.gens + ((size_t)k * a.G + g) * NN + idx) * coef[k * a.G + g], m1, acc);
                    }
                }
                X[idx] = acc;
            }
            __syncthreads();
            double* Eout;  // the exponential (residual form if a.residual)
            if (a.expm == SSS_EXPM_REFERENCE) {
                // :534-578 scale and (non-residual) shift; :882-897 squarings
                double scale = ldexp(1.0, 2 * a.R);
                for (int idx = threadIdx.x; idx < NN; idx += blockDim.x) {
                    double v = X[idx] / scale;
                    if (!a.residual && idx / N == idx % N) v += 1.0;
                    X[idx] = v;
                }
                __syncthreads();
                for (int q = 0; q < a.R; q++) {
                    mm_ref(X2, X, X, N, true, a.residual);
                    __syncthreads();
                    mm_ref(X, X2, X2, N, true, a.residual);
                    __syncthreads();
                }
                Eout = X;
            } else {
                // scaling: ||X||_1 <= 0.25 * 2^s  (Taylor-12 truncation < 1e-18)
                if (threadIdx.x < N) {
                    double s = 0.0;
                    for (int i = 0; i < N; i++) s += fabs(X[i * N + threadIdx.x]);
                    colsum[threadIdx.x] = s;
                }
                __syncthreads();
                double nrm = 0.0;
                for (int j = 0; j < N; j++) nrm = fmax(nrm, colsum[j]);
                int s = 0;
                while (nrm > 0.25 && s < 60) { nrm *= 0.5; s++; }
                if (s > 0) {
                    double f = ldexp(1.0, -s);
                    for (int idx = threadIdx.x; idx < NN; idx += blockDim.x) X[idx] *= f;
                    __syncthreads();
                }
                // Paterson-Stockmeyer, E = sum_{j=1..12} X^j/j!
                const double c[13] = {1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720,
                                      1.0 / 5040, 1.0 / 40320, 1.0 / 362880, 1.0 / 3628800,
                                      1.0 / 39916800, 1.0 / 479001600};
                mm(X2, X, X, N, 0, 0);
                __syncthreads();
                mm(X3, X2, X, N, 0, 0);
                mm(X4, X2, X2, N, 0, 0);
                __syncthreads();
                for (int idx = threadIdx.x; idx < NN; idx += blockDim.x)
                    Bm[idx] = (idx / N == idx % N ? c[8] : 0.0) + c[9] * X[idx] + c[10] * X2[idx] +
                              c[11] * X3[idx] + c[12] * X4[idx];
                __syncthreads();
                mm(E, X4, Bm, N, 0, 0);
                __syncthreads();
                for (int idx = threadIdx.x; idx < NN; idx += blockDim.x)
                    E[idx] += (idx / N == idx % N ? c[4] : 0.0) + c[5] * X[idx] + c[6] * X2[idx] +
                              c[7] * X3[idx];
                __syncthreads();
                mm(Bm, X4, E, N, 0, 0);
                __syncthreads();
                for (int idx = threadIdx.x; idx < NN; idx += blockDim.x)
                    Bm[idx] += c[1] * X[idx] + c[2] * X2[idx] + c[3] * X3[idx];
                __syncthreads();
                double* cur = Bm;
                double* nxt = E;
                for (int q = 0; q < s; q++) {  // residual squaring: 2E + E^2
                    mm(nxt, cur, cur, N, 2.0, 0.0);
                    __syncthreads();
                    double* tmp = cur; cur = nxt; nxt = tmp;
                }
                if (!a.residual) {
                    for (int idx = threadIdx.x; idx < NN; idx += blockDim.x)
                        if (idx / N == idx % N) cur[idx] += 1.0;
                    __syncthreads();
                }
                Eout = cur;
            }
            // TE <- E (*) TE  (:726-743, :1259-1294)
            if (a.expm == SSS_EXPM_REFERENCE)
                mm_ref(T2, Eout, TE, N, false, a.residual);
            else
                mm(T2, Eout, TE, N, a.residual ? 1.0 : 0.0, a.residual ? 1.0 : 0.0);
            __syncthreads();
            double* tmp = TE; TE = T2; T2 = tmp;
        }
        if (a.rotating) {
            // :901-964 -- TE <- e^{L0 h} TE with residual-aware blocks
            for (int idx = threadIdx.x; idx < NN; idx += blockDim.x) {
                int y = idx / N, x = idx - y * N;
                double v;
                if (y < 2 * a.D) {
                    int blk = y >> 1;
                    double p = a.dlast[2 * blk], q = a.dlast[2 * blk + 1];
                    double re_in = TE[(2 * blk) * N + x], im_in = TE[(2 * blk + 1) * N + x];
                    if (a.residual) {
                        if ((y & 1) == 0) {
                            v = (1 + p) * re_in - q * im_in;
                            if (x == 2 * blk) v += p;
                            if (x == 2 * blk + 1) v -= q;
                        } else {
                            v = q * re_in + (1 + p) * im_in;
                            if (x == 2 * blk) v += q;
                            if (x == 2 * blk + 1) v += p;
                        }
                    } else {
                        v = ((y & 1) == 0) ? p * re_in - q * im_in : q * re_in + p * im_in;
                    }
                } else {
                    double s = a.slast[y - 2 * a.D];
                    if (a.residual) {
                        v = (1 + s) * TE[idx];
                        if (y == x) v += s;
                    } else {
                        v = s * TE[idx];
                    }
                }
                T2[idx] = v;
            }
            __syncthreads();
            double* tmp = TE; TE = T2; T2 = tmp;
        }
    }
    __syncthreads();
    double* dst = a.out + ((size_t)b * a.T + t) * NN;
    for (int idx = threadIdx.x; idx < NN; idx += blockDim.x) dst[idx] = TE[idx];
}

// v <- v + S v (residual) or S v, for t = 0..T-1; writes out[b][t] (lab basis).
// With an image basis P (n_full x N, equivalence-class mode): the chain runs
// on x0 = P^T rho0 and the output is rho0 + P (y - x0), y the chain's lab-basis
// vector -- the full propagator P (I + E) P^T + (I - P P^T): components in the
// generators' common kernel stay fixed (the intended form of the reference's
// sandwich and kernel addition, generate_simulator.py:2043-2071).
// state[b] holds the running vector between chunks (in the eigenbasis when
// rotating), followed by x0 when projecting.
__global__ void __launch_bounds__(kPlainThreads)
k_chain(const double* __restrict__ S, const double* __restrict__ rho0, const double* __restrict__ V,
        const double* __restrict__ Vinv, const double* __restrict__ P, int n_full, int N, int T,
        int residual, int t_begin, double* __restrict__ state, double* __restrict__ out) {
    __shared__ double v[kPlainMaxN], w[kPlainMaxN], x0[kPlainMaxN], y[kPlainMaxN];
    const int b = blockIdx.x, NN = N * N;
    const int nio = P ? n_full : N;  // entries of a state in and of a sample out
    const int sw = P ? 2 * N : N;    // state words per trajectory
    if (t_begin == 0) {
        if (threadIdx.x < N) {
            double acc = 0.0;
            if (P) {
                for (int k = 0; k < n_full; k++)
                    acc = fma(P[(size_t)k * N + threadIdx.x], rho0[(size_t)b * nio + k], acc);
            } else {
                acc = rho0[(size_t)b * N + threadIdx.x];
            }
            x0[threadIdx.x] = acc;
        }
        __syncthreads();
        if (threadIdx.x < N) {
            double acc = x0[threadIdx.x];
            if (Vinv) {
                acc = 0.0;
                for (int k = 0; k < N; k++) acc = fma(Vinv[threadIdx.x * N + k], x0[k], acc);
            }
            v[threadIdx.x] = acc;
        }
    } else if (threadIdx.x < N) {
        v[threadIdx.x] = state[(size_t)b * sw + threadIdx.x];
        if (P) x0[threadIdx.x] = state[(size_t)b * sw + N + threadIdx.x];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int t = 0; t < T; t++) {
        const double* St = S + ((size_t)b * T + t) * NN;
        for (int i = warp; i < N; i += nw) {
            double acc = 0.0;
            for (int k = lane; k < N; k += 32) acc = fma(__ldg(St + i * N + k), v[k], acc);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) w[i] = residual ? v[i] + acc : acc;
        }
        __syncthreads();
        if (threadIdx.x < N) v[threadIdx.x] = w[threadIdx.x];
        __syncthreads();
        if (threadIdx.x < N) {
            double o = v[threadIdx.x];
            if (V) {
                o = 0.0;
                for (int k = 0; k < N; k++) o = fma(V[threadIdx.x * N + k], v[k], o);
            }
            y[threadIdx.x] = o;
        }
        __syncthreads();
        double* ot = out + (size_t)(t_begin + t) * nio;
        if (!P) {
            if (threadIdx.x < N) ot[threadIdx.x] = y[threadIdx.x];
        } else {
            for (int i = threadIdx.x; i < n_full; i += blockDim.x) {
                double acc = rho0[(size_t)b * nio + i];
                for (int k = 0; k < N; k++) acc = fma(P[(size_t)i * N + k], y[k] - x0[k], acc);
                ot[i] = acc;
            }
        }
    }
    if (threadIdx.x < N) {
        state[(size_t)b * sw + threadIdx.x] = v[threadIdx.x];
        if (P) state[(size_t)b * sw + N + threadIdx.x] = x0[threadIdx.x];
    }
}

// Unitary mode (generate_simulator.py:2074-2101 with :1394-1504): the step
// propagators act on a u_n-level operator in real 2n x 2n form (entry (i, j)
// of the complex matrix at [2i][2j] real, [2i+1][2j] imaginary).  One CTA per
// trajectory keeps the running operator propagator M (M - I in residual
// form; in the eigenbasis when rotating, U = V M V^-1), and after every
// sample writes the density conj(U) rho0 U^T -- what the reference's
// Kronecker product, unitary copy and elimination/duplication sandwich give
// -- in the basis of the vectorisation map (rows y, x, c as doubles), or all
// 2n^2 entries row-major.  state[b] holds M between chunks.
__global__ void __launch_bounds__(kPlainThreads)
k_chain_unitary(const double* __restrict__ S, const double* __restrict__ rho0,
                const double* __restrict__ V, const double* __restrict__ Vinv,
                const double* __restrict__ umap, int n, int nd, int T, int residual, int t_begin,
                double* __restrict__ state, double* __restrict__ out) {
    extern __shared__ double sm[];
    const int D = 2 * n, DD = D * D, nn = n * n;
    double* M = sm;           // D x D
    double* A = M + DD;       // D x D scratch
    double* U = A + DD;       // D x D lab-basis propagator
    double* r0 = U + DD;      // n x n complex rho0 (re, im interleaved)
    double* tm = r0 + 2 * nn; // n x n complex conj(U) rho0
    const int b = blockIdx.x;
    auto map_row = [&](int i, int* y, int* x, int* c) {
        if (umap) {
            *y = (int)umap[3 * i];
            *x = (int)umap[3 * i + 1];
            *c = (int)umap[3 * i + 2];
        } else {
            *y = (i >> 1) / n;
            *x = (i >> 1) % n;
            *c = i & 1;
        }
    };
    for (int i = threadIdx.x; i < 2 * nn; i += blockDim.x) r0[i] = 0.0;
    __syncthreads();
    if (threadIdx.x == 0) {
        // rho0 from its flattened form; mapped off-diagonal entries mirror
        // to the Hermitian partner
        for (int i = 0; i < nd; i++) {
            int y, x, c;
            map_row(i, &y, &x, &c);
            const double val = rho0[(size_t)b * nd + i];
            r0[2 * (y * n + x) + c] = val;
            if (umap && y != x) r0[2 * (x * n + y) + c] = c ? -val : val;
        }
    }
    for (int i = threadIdx.x; i < DD; i += blockDim.x)
        M[i] = t_begin == 0 ? ((!residual && i / D == i % D) ? 1.0 : 0.0) : state[(size_t)b * DD + i];
    __syncthreads();
    for (int t = 0; t < T; t++) {
        const double* Et = S + ((size_t)b * T + t) * DD;
        // M <- (I + E) M - I = E + M + E M (residual), or E M
        for (int idx = threadIdx.x; idx < DD; idx += blockDim.x) {
            const int i = idx / D, j = idx - i * D;
            double acc = residual ? __ldg(Et + idx) + M[idx] : 0.0;
            for (int k = 0; k < D; k++) acc = fma(__ldg(Et + i * D + k), M[k * D + j], acc);
            A[idx] = acc;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < DD; idx += blockDim.x) M[idx] = A[idx];
        __syncthreads();
        // U (lab basis) = V (I + M) V^-1, or I + M
        if (V) {
            for (int idx = threadIdx.x; idx < DD; idx += blockDim.x) {
                const int i = idx / D, j = idx - i * D;
                double acc = residual ? Vinv[idx] : 0.0;
                for (int k = 0; k < D; k++) acc = fma(M[i * D + k], Vinv[k * D + j], acc);
                A[idx] = acc;
            }
            __syncthreads();
            for (int idx = threadIdx.x; idx < DD; idx += blockDim.x) {
                const int i = idx / D, j = idx - i * D;
                double acc = 0.0;
                for (int k = 0; k < D; k++) acc = fma(V[i * D + k], A[k * D + j], acc);
                U[idx] = acc;
            }
        } else {
            for (int idx = threadIdx.x; idx < DD; idx += blockDim.x)
                U[idx] = M[idx] + ((residual && idx / D == idx % D) ? 1.0 : 0.0);
        }
        __syncthreads();
        // tm = conj(Uc) rho0, Uc[i][k] = U[2i][2k] + i U[2i+1][2k]
        for (int idx = threadIdx.x; idx < nn; idx += blockDim.x) {
            const int i = idx / n, j = idx - i * n;
            double re = 0.0, im = 0.0;
            for (int k = 0; k < n; k++) {
                const double ur = U[(2 * i) * D + 2 * k], ui = -U[(2 * i + 1) * D + 2 * k];
                const double rr = r0[2 * (k * n + j)], ri = r0[2 * (k * n + j) + 1];
                re = fma(ur, rr, re);
                re = fma(-ui, ri, re);
                im = fma(ur, ri, im);
                im = fma(ui, rr, im);
            }
            tm[2 * idx] = re;
            tm[2 * idx + 1] = im;
        }
        __syncthreads();
        // rho = tm Uc^T: rho[y][x] = sum_k tm[y][k] Uc[x][k]; write the mapped entries
        double* ot = out + (size_t)(t_begin + t) * nd;
        for (int i = threadIdx.x; i < nd; i += blockDim.x) {
            int y, x, c;
            map_row(i, &y, &x, &c);
            double re = 0.0, im = 0.0;
            for (int k = 0; k < n; k++) {
                const double ur = U[(2 * x) * D + 2 * k], ui = U[(2 * x + 1) * D + 2 * k];
                const double tr = tm[2 * (y * n + k)], ti = tm[2 * (y * n + k) + 1];
                re = fma(tr, ur, re);
                re = fma(-ti, ui, re);
                im = fma(tr, ui, im);
                im = fma(ti, ur, im);
            }
            ot[i] = c ? im : re;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < DD; i += blockDim.x) state[(size_t)b * DD + i] = M[i];
}

}  // namespace

int plain_run(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg,
              const double* d_prog, const double* d_tab, double t0, double dt,
              int T, int F, double* d_out, cudaStream_t st) {
    const int N = p->d.N;
    if (N > kPlainMaxN)
        return fail(SSS_EINVAL, "plain path supports N <= 52 (got " + std::to_string(N) + ")");
    const size_t NN = (size_t)N * N;
    // Chunk the samples so the step-propagator buffer stays under ~2 GiB.
    size_t per_sample = NN * sizeof(double);
    int chunk = (int)std::min<size_t>((size_t)T, std::max<size_t>(1, (2ull << 30) / per_sample));
    if (int rc = p->w_prop.ensure(per_sample * (size_t)chunk)) return rc;
    const int nio = p->state_in();  // entries of a state in and of a sample out
    if (int rc = p->w_aux.ensure(sizeof(double) * (p->u_n ? NN : 2 * (size_t)N))) return rc;
    const size_t usmem = sizeof(double) * (3 * NN + 4 * (size_t)p->u_n * p->u_n);
    if (p->u_n)
        SSS_CUDA(cudaFuncSetAttribute(k_chain_unitary, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)usmem));
    size_t smem = 8 * NN * sizeof(double);
    SSS_CUDA(cudaFuncSetAttribute(k_step_propagators, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    int launches = 0;
    for (int b = 0; b < ntraj; b++) {
        for (int t_begin = 0; t_begin < T; t_begin += chunk) {
            int Tc = std::min(chunk, T - t_begin);
            PlainArgs a{};
            a.N = N; a.G = p->d.G; a.K = p->d.K; a.Q = p->d.Q; a.F = F; a.T = Tc;
            a.nch = nch; a.nseg = nseg; a.expm = p->d.expm; a.R = p->d.quartic_repeats;
            a.residual = (p->d.flags & SSS_RESIDUAL) != 0;
            a.rotating = p->rotating;
            a.gens = p->d_gens.as<double>();
            a.W = p->d_gens.as<double>() + p->gens.size();  // W and nodes follow the generators
            a.nodes = a.W + p->d.K * p->d.Q;
            a.dlast = p->d_dlast.as<double>(); a.slast = p->d_slast.as<double>();
            a.D = p->D; a.S = p->S;
            a.prog = d_prog ? d_prog + (size_t)b * nch * nseg * 5 : nullptr;
            a.tab = nullptr;
            a.t0 = t0;
            a.dt = dt;
            a.t_offset = t_begin;
            a.out = p->w_prop.as<double>();
            if (d_tab) {
                // copy this chunk's rows (r, t, k) of the table, in order
                size_t rowG = (size_t)p->d.Q * p->d.G;
                if (int rc = p->w_tab.ensure(sizeof(double) * (size_t)F * Tc * rowG)) return rc;
                const double* src = d_tab + (size_t)b * F * T * rowG;
                SSS_CUDA(cudaMemcpy2DAsync(p->w_tab.p, Tc * rowG * sizeof(double),
                                           src + (size_t)t_begin * rowG, (size_t)T * rowG * sizeof(double),
                                           Tc * rowG * sizeof(double), F, cudaMemcpyDeviceToDevice, st));
                a.tab = p->w_tab.as<double>();
            }
            dim3 grid(Tc, 1);
            k_step_propagators<<<grid, kPlainThreads, smem, st>>>(a);
            launches++;
            SSS_CUDA(cudaGetLastError());
            const double* V = p->rotating ? p->d_V.as<double>() : nullptr;
            const double* Vi = p->rotating ? p->d_Vinv.as<double>() : nullptr;
            if (p->u_n)
                k_chain_unitary<<<1, kPlainThreads, usmem, st>>>(
                    p->w_prop.as<double>(), d_rho0 + (size_t)b * nio, V, Vi,
                    p->u_mapped ? p->d_umap.as<double>() : nullptr, p->u_n, p->u_nd, Tc,
                    a.residual ? 1 : 0, t_begin, p->w_aux.as<double>(), d_out + (size_t)b * T * nio);
            else
                k_chain<<<1, kPlainThreads, 0, st>>>(
                    p->w_prop.as<double>(), d_rho0 + (size_t)b * nio, V, Vi,
                    p->n_full ? p->d_P.as<double>() : nullptr, p->n_full, N, Tc,
                    a.residual ? 1 : 0, t_begin, p->w_aux.as<double>(), d_out + (size_t)b * T * nio);
            launches++;
            SSS_CUDA(cudaGetLastError());
        }
    }
    p->last_launches = launches;
    return SSS_OK;
}

}  // namespace sss

// ---------------------------------------------------------------------------
// Allocation-free variant of the plain path.
//
// Some callers cannot allocate device memory: code running inside another
// framework's memory pool (which would fragment or be bypassed), callers
// on a device whose memory is already fully reserved, or callers whose own
// rules forbid allocation while they run.  sss_simulate_noalloc runs the
// same two kernels as sss_simulate_device for one trajectory in the lab
// frame, but instead of a plan's buffers it uses one file-scope device
// array as its scratch: the weight/node table, the chain's running state
// and a chunk of step propagators.  It allocates nothing on the device or
// the host, and it copies nothing from host memory: the weight/node table
// reaches the scratch as a kernel argument.
//
// Limits: N <= 52 (the shared-memory path), lab frame only, and the
// step-propagator chunk must hold at least one N x N matrix (always true
// for N <= 52).  The array is 4 MiB; every GPU that loads this library
// keeps it until the process exits.  Every call shares it and it keeps the
// last call's contents, so calls that overlap on the GPU (on different
// streams, or from different host threads) race and corrupt each other.
// The first call on a device looks up the array's device address on that
// device; make that first call before any stream capture.  Every call sets
// the step kernel's shared-memory limit for its own N (other entry points
// of the library set the same per-function limit for theirs).
// ---------------------------------------------------------------------------

namespace sss {
namespace {

constexpr size_t kNoallocBytes = 4u << 20;
constexpr int kNoallocMaxDevices = 64;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

struct NoallocDevice {
    double* ptr = nullptr;
    bool ready = false;
};
static NoallocDevice g_noalloc_dev[kNoallocMaxDevices];
static std::mutex g_noalloc_mutex;

// Device address of the scratch array on the current device (set up once
// per device, with that device current).
int noalloc_scratch(double** out) {
    int dev = 0;
    SSS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoallocMaxDevices) return fail(SSS_EINVAL, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoallocDevice& d = g_noalloc_dev[dev];
    if (!d.ready) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
        d.ptr = static_cast<double*>(ptr);
        d.ready = true;
    }
    *out = d.ptr;
    return SSS_OK;
}

// The CF weights (K*Q) then the nodes (Q), passed by value.
struct NoallocTable {
    double v[kMaxK * kMaxQ + kMaxQ];
    int n;
};

__global__ void k_noalloc_table(const NoallocTable t, double* __restrict__ dst) {
    for (int i = threadIdx.x; i < t.n; i += blockDim.x) dst[i] = t.v[i];
}

}  // namespace
}  // namespace sss

extern "C" int sss_simulate_noalloc(const sss_plan_desc* d, const double* generators,
                                    const double* weights, const double* nodes,
                                    const double* rho0, int nch, int nseg,
                                    const double* programs, double t0, double dt, int T, int F,
                                    double* out, void* stream) {
    using namespace sss;
    if (!d) return fail(SSS_EINVAL, "null descriptor");
    const int N = d->N;
    if (N <= 0 || N > kPlainMaxN)
        return fail(SSS_EINVAL, "sss_simulate_noalloc supports 1 <= N <= 52 (got " +
                                    std::to_string(N) + ")");
    if (d->G <= 0 || d->G > kMaxG || d->K <= 0 || d->K > kMaxK || d->Q <= 0 || d->Q > kMaxQ)
        return fail(SSS_EINVAL, "bad plan shape (G, K, Q)");
    if (d->flags & SSS_ROTATING) return fail(SSS_EINVAL, "sss_simulate_noalloc is lab-frame only");
    if (d->expm != SSS_EXPM_REFERENCE && d->expm != SSS_EXPM_TAYLOR)
        return fail(SSS_EINVAL, "unknown exponential algorithm");
    if (d->expm == SSS_EXPM_REFERENCE && (d->quartic_repeats < 0 || d->quartic_repeats > 500))
        return fail(SSS_EINVAL, "quartic_repeats out of range");
    if (T < 0 || F <= 0) return fail(SSS_EINVAL, "bad T or F");
    if (T == 0) return SSS_OK;
    if (!generators || !weights || !nodes || !rho0 || !programs || !out)
        return fail(SSS_EINVAL, "null argument");
    if (nch < 0 || nch > kMaxCh || nseg <= 0) return fail(SSS_EINVAL, "bad program shape");
    if (!(dt > 0) || !std::isfinite(dt)) return fail(SSS_EINVAL, "dt must be positive and finite");

    double* scratch = nullptr;
    if (int rc = noalloc_scratch(&scratch)) return rc;
    // layout: [0, 32) weights then nodes; [32, 96) chain state; then step
    // propagators
    const size_t NN = (size_t)N * N;
    double* wn = scratch;
    double* chain_state = scratch + 32;
    double* props = scratch + 96;
    const size_t prop_capacity = (kNoallocBytes / sizeof(double) - 96) / NN;
    if (prop_capacity < 1) return fail(SSS_EINVAL, "scratch too small for one propagator");
    const int chunk = (int)std::min<size_t>((size_t)T, prop_capacity);

    cudaStream_t st = (cudaStream_t)stream;
    NoallocTable tbl{};
    tbl.n = d->K * d->Q + d->Q;
    for (int i = 0; i < d->K * d->Q; i++) tbl.v[i] = weights[i];
    for (int k = 0; k < d->Q; k++) tbl.v[d->K * d->Q + k] = nodes[k];
    k_noalloc_table<<<1, 32, 0, st>>>(tbl, wn);
    SSS_CUDA(cudaGetLastError());
    // the limit is per function and per device, and the plan entry points
    // set it for their own N, so it is set here on every call
    const size_t smem = 8 * NN * sizeof(double);
    SSS_CUDA(cudaFuncSetAttribute(k_step_propagators, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    for (int t_begin = 0; t_begin < T; t_begin += chunk) {
        int Tc = std::min(chunk, T - t_begin);
        PlainArgs a{};
        a.N = N; a.G = d->G; a.K = d->K; a.Q = d->Q; a.F = F; a.T = Tc;
        a.nch = nch; a.nseg = nseg; a.expm = d->expm; a.R = d->quartic_repeats;
        a.t_offset = t_begin;
        a.residual = (d->flags & SSS_RESIDUAL) != 0;
        a.rotating = false;
        a.gens = generators;
        a.W = wn;
        a.nodes = wn + d->K * d->Q;
        a.prog = programs;
        a.tab = nullptr;
        a.t0 = t0;
        a.dt = dt;
        a.out = props;
        k_step_propagators<<<dim3(Tc, 1), kPlainThreads, smem, st>>>(a);
        SSS_CUDA(cudaGetLastError());
        k_chain<<<1, kPlainThreads, 0, st>>>(props, rho0, nullptr, nullptr, nullptr, 0, N, Tc,
                                             a.residual ? 1 : 0, t_begin, chain_state, out);
        SSS_CUDA(cudaGetLastError());
    }
    return SSS_OK;
}
