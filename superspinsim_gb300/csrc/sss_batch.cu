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
//     v <- v + sum_{j=1..d} Omega^j v / j!   (m sub-steps of Omega/m),
// with d and m chosen from a norm bound so the truncation stays below
// 1e-18 per exponential.  Omega = h * sum_g a_g G_g is assembled only on
// the union sparsity pattern of the generators, restricted to the state
// entries reachable from the initial states' support (entries outside it
// are exact zeros for all time and are skipped, so results are unchanged).
//
// Layout: a "group" of L lanes (one warp or a fraction of one) owns one
// trajectory at a time; its rows are split across the L lanes, balanced by
// non-zeros.  Generator values, the CSR pattern and readout weights are
// staged in shared memory once per CTA; per-group state (assembled Omega,
// state vector, Taylor terms, coefficients) lives in shared memory.  Groups
// take trajectories from a global atomic counter (the device work queue)
// and keep going until it is exhausted, so uneven trajectory lengths
// balance across the GPU.  The step loop is flat -- finishing a trajectory
// and loading the next is a short branch inside it -- so the groups of a
// warp stay converged in the arithmetic.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "sss_device.cuh"
#include "sss_internal.cuh"

namespace sss {

// ---------------------------------------------------------------------------
// host: sparse pattern
// ---------------------------------------------------------------------------

int build_sparse(sss_plan* p) {
    const int N = p->d.N, G = p->d.G;
    SparseGenerators& s = p->sparse;
    s.N = N;
    s.G = G;
    s.row_ptr.assign(N + 1, 0);
    s.col.clear();
    std::vector<std::vector<double>> vals(G);
    for (int r = 0; r < N; r++) {
        for (int c = 0; c < N; c++) {
            bool nz = false;
            for (int g = 0; g < G; g++)
                if (p->gens[((size_t)g * N + r) * N + c] != 0.0) nz = true;
            if (!nz) continue;
            s.col.push_back(c);
            for (int g = 0; g < G; g++) vals[g].push_back(p->gens[((size_t)g * N + r) * N + c]);
        }
        s.row_ptr[r + 1] = (int)s.col.size();
    }
    s.nnz = (int)s.col.size();
    s.val.clear();
    for (int g = 0; g < G; g++) s.val.insert(s.val.end(), vals[g].begin(), vals[g].end());
    return SSS_OK;
}

namespace {

constexpr int kMaxTaylor = 24;

struct BatchArgs {
    int M, G, K, Q, F, nch, nseg, T_max, ntraj, degree, substeps;
    int nnz;
    double h_sub, t0, dt;
    const double* toff;      // F: (r*dt)/F, rounded as the reference rounds it
    const double* noff;      // Q: (dt*node_k)/F
    const double* W;         // K*Q
    const double* nodes;     // Q
    const int* rows;         // M+1 CSR row pointer (compressed, lane-ordered)
    const int* cols;         // nnz (compressed column index)
    const double* vals;      // G*nnz
    const int* lane_rows;    // L+1: rows [lane_rows[l], lane_rows[l+1]) belong to lane l
    const int* row_orig;     // M: original index of compressed row
    const double* rw;        // M readout weights (compressed), or null
    const double* rho0;      // ntraj*N
    const double* prog;      // ntraj*nch*nseg*5
    const int* samples;      // ntraj or null
    int N;
    double* readout;         // ntraj*T_max or null
    double* fin;             // ntraj*N or null
    int* queue;              // work counter
    double inv_j[kMaxTaylor + 1];
};

template <int L>
__global__ void __launch_bounds__(256) k_batch(const BatchArgs a) {
    extern __shared__ double smem[];
    const int M = a.M, nnz = a.nnz, G = a.G;
    // CTA-shared staging
    double* s_val = smem;                              // G*nnz
    double* s_rw = s_val + (size_t)G * nnz;            // M
    int* s_rows = reinterpret_cast<int*>(s_rw + M);    // M+1
    int* s_cols = s_rows + (M + 1);                    // nnz
    int* s_lane = s_cols + nnz;                        // L+1
    size_t shared_words = (size_t)G * nnz + M + ((M + 1 + nnz + L + 1 + 1) / 2);
    double* slots = smem + shared_words;
    const int slot = threadIdx.x / L, li = threadIdx.x % L;
    const int per_slot = nnz + 4 * M + kMaxQ * kMaxG;
    double* Om = slots + (size_t)slot * per_slot;
    double* v = Om + nnz;
    double* term = v + M;
    double* nxt = term + M;
    double* acc = nxt + M;
    double* coef = acc + M;

    for (int i = threadIdx.x; i < G * nnz; i += blockDim.x) s_val[i] = a.vals[i];
    for (int i = threadIdx.x; i < M; i += blockDim.x) s_rw[i] = a.rw ? a.rw[i] : 0.0;
    for (int i = threadIdx.x; i <= M; i += blockDim.x) s_rows[i] = a.rows[i];
    for (int i = threadIdx.x; i < nnz; i += blockDim.x) s_cols[i] = a.cols[i];
    for (int i = threadIdx.x; i <= L; i += blockDim.x) s_lane[i] = a.lane_rows[i];
    __syncthreads();

    const unsigned lane_in_warp = threadIdx.x & 31;
    const unsigned gmask = (L == 32) ? 0xffffffffu
                                     : (((1u << L) - 1u) << (lane_in_warp / L * L));
    const int r_begin = s_lane[li], r_end = s_lane[li + 1];

    int b = -1, T_b = 0, t = 0, r = 0;
    const double* prog = nullptr;
    // Flat loop: one iteration = one fine step of the group's trajectory.
    while (true) {
        if (r == 0 && t >= T_b) {
            // finish the current trajectory, take the next one
            if (b >= 0 && a.fin) {
                for (int i = r_begin; i < r_end; i++) a.fin[(size_t)b * a.N + a.row_orig[i]] = v[i];
            }
            int nb = 0;
            if (li == 0) nb = atomicAdd(a.queue, 1);
            nb = __shfl_sync(gmask, nb, lane_in_warp / L * L);
            b = nb;
            if (b >= a.ntraj) break;
            T_b = a.samples ? a.samples[b] : a.T_max;
            t = 0;
            prog = a.prog + (size_t)b * a.nch * a.nseg * 5;
            for (int i = r_begin; i < r_end; i++) v[i] = a.rho0[(size_t)b * a.N + a.row_orig[i]];
            __syncwarp(gmask);
            if (T_b == 0) continue;
        }
        // coefficients at the Q nodes: [1, ch0, ch1, ...] (lab frame)
        for (int i = li; i < a.Q * G; i += L) {
            int k = i / G, g = i - k * G;
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
        __syncwarp(gmask);
        for (int e = a.K - 1; e >= 0; e--) {
            double ag[kMaxG];
            for (int g = 0; g < G; g++) {
                double s = 0.0;
                for (int k = 0; k < a.Q; k++) s = fma(a.W[e * a.Q + k], coef[k * G + g], s);
                ag[g] = s * a.h_sub;
            }
            // assemble Omega on my rows' entries
            for (int p = s_rows[r_begin]; p < s_rows[r_end]; p++) {
                double o = 0.0;
                for (int g = 0; g < G; g++) o = fma(ag[g], s_val[(size_t)g * nnz + p], o);
                Om[p] = o;
            }
            for (int m = 0; m < a.substeps; m++) {
                for (int i = r_begin; i < r_end; i++) {
                    term[i] = v[i];
                    acc[i] = 0.0;
                }
                __syncwarp(gmask);
                double* cur = term;
                double* nx = nxt;
                for (int j = 1; j <= a.degree; j++) {
                    for (int i = r_begin; i < r_end; i++) {
                        double s = 0.0;
                        for (int p = s_rows[i]; p < s_rows[i + 1]; p++) s = fma(Om[p], cur[s_cols[p]], s);
                        s *= a.inv_j[j];
                        nx[i] = s;
                        acc[i] += s;
                    }
                    __syncwarp(gmask);
                    double* tmp = cur; cur = nx; nx = tmp;
                }
                for (int i = r_begin; i < r_end; i++) v[i] += acc[i];
                __syncwarp(gmask);
            }
        }
        if (++r == a.F) {
            r = 0;
            if (a.readout) {
                double s = 0.0;
                for (int i = r_begin; i < r_end; i++) s = fma(s_rw[i], v[i], s);
#pragma unroll
                for (int o = L / 2; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
                if (li == 0) a.readout[(size_t)b * a.T_max + t] = s;
            }
            t++;
        }
    }
}

template <int L>
int launch_batch(sss_plan* p, const BatchArgs& a, int threads, size_t smem, cudaStream_t st) {
    SSS_CUDA(cudaFuncSetAttribute(k_batch<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    SSS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<L>, threads, smem));
    if (per_sm < 1) return fail(SSS_EINVAL, "batched kernel does not fit on an SM");
    int slots_per_cta = threads / L;
    int want = (a.ntraj + slots_per_cta - 1) / slots_per_cta;
    int grid = std::max(1, std::min(want, per_sm * p->num_sms));
    if (!p->ev_begin) {
        SSS_CUDA(cudaEventCreate(&p->ev_begin));
        SSS_CUDA(cudaEventCreate(&p->ev_end));
    }
    SSS_CUDA(cudaEventRecord(p->ev_begin, st));
    k_batch<L><<<grid, threads, smem, st>>>(a);
    SSS_CUDA(cudaGetLastError());
    SSS_CUDA(cudaEventRecord(p->ev_end, st));
    p->ev_recorded = true;
    return SSS_OK;
}

}  // namespace

// Taylor degree and sub-steps for a norm bound `beta` of Omega: the
// smallest d*m with m*(beta/m)^(d+1)/(d+1)! <= 1e-18.
static void choose_taylor(double beta, int forced_degree, int* degree, int* substeps) {
    if (forced_degree > 0) {
        *degree = std::min(forced_degree, kMaxTaylor);
        int m = 1;
        while (m < 1024) {
            double x = beta / m, term = 1.0;
            for (int j = 1; j <= *degree + 1; j++) term *= x / j;
            if (m * term <= 1e-18) break;
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
            if (m * next <= 1e-18) {
                if (d * m < best_d * best_m) { best_d = d; best_m = m; }
                break;
            }
        }
        if (best_d * best_m <= m) break;
    }
    *degree = best_d;
    *substeps = best_m;
}

int batch_run(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg, const double* d_prog,
              const int* d_samples, const int* h_samples, double t0, double dt, int T_max, int F,
              const double* h_rw, double* d_readout, double* d_final, cudaStream_t st) {
    (void)h_samples;
    const int N = p->d.N, G = p->d.G;
    const SparseGenerators& sp = p->sparse;
    // ---- reachable rows from the initial states' support ----
    std::vector<double> h_rho0((size_t)ntraj * N);
    SSS_CUDA(cudaMemcpyAsync(h_rho0.data(), d_rho0, sizeof(double) * h_rho0.size(), cudaMemcpyDeviceToHost, st));
    SSS_CUDA(cudaStreamSynchronize(st));
    std::vector<char> reach(N, 0);
    std::vector<int> stack;
    for (int b = 0; b < ntraj; b++)
        for (int i = 0; i < N; i++)
            if (h_rho0[(size_t)b * N + i] != 0.0 && !reach[i]) { reach[i] = 1; stack.push_back(i); }
    // column c influences row r when (r, c) is in the pattern
    std::vector<std::vector<int>> influences(N);
    for (int r = 0; r < N; r++)
        for (int q = sp.row_ptr[r]; q < sp.row_ptr[r + 1]; q++) influences[sp.col[q]].push_back(r);
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
    if (d_readout) SSS_CUDA(cudaMemsetAsync(d_readout, 0, sizeof(double) * (size_t)ntraj * T_max, st));
    if (d_final) SSS_CUDA(cudaMemsetAsync(d_final, 0, sizeof(double) * (size_t)ntraj * N, st));
    if (M == 0) { p->last_launches = 0; return SSS_OK; }

    // ---- lanes per trajectory (autotuned choice comes from the caller's
    // table; default from the problem size) ----
    // Lanes per trajectory: FP64 on GB300 issues ~2 DFMA/clk/SM with a
    // 75-cycle latency, so each SM wants >= 16 warps of dependent chains.
    // Take the fewest lanes that give that many lanes in flight, capped by
    // the rows available to split.
    int L = 1;
    {
        const long want = (long)p->num_sms * 16 * 32;
        int cap = 1;
        while (cap < 32 && cap * 2 <= std::max(1, M)) cap *= 2;
        while (L < cap && (long)ntraj * L < want) L *= 2;
    }
    if (p->batch_lanes > 0) L = p->batch_lanes;
    // ---- assign rows to lanes balanced by non-zeros; relabel compressed
    // rows so that each lane's rows are contiguous ----
    std::vector<int> nz_of(M);
    for (int i = 0; i < M; i++) {
        int r = rows_reached[i], c = 0;
        for (int q = sp.row_ptr[r]; q < sp.row_ptr[r + 1]; q++) c += reach[sp.col[q]] ? 1 : 0;
        nz_of[i] = c + 2;  // + per-row overhead
    }
    std::vector<int> order(M);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return nz_of[x] > nz_of[y]; });
    std::vector<long> load(L, 0);
    std::vector<std::vector<int>> lane_of(L);
    for (int i : order) {
        int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[l] += nz_of[i];
        lane_of[l].push_back(i);
    }
    std::vector<int> newpos(M), row_orig(M), lane_rows(L + 1, 0);
    {
        int k = 0;
        for (int l = 0; l < L; l++) {
            std::sort(lane_of[l].begin(), lane_of[l].end());
            for (int i : lane_of[l]) { newpos[i] = k; row_orig[k] = rows_reached[i]; k++; }
            lane_rows[l + 1] = k;
        }
    }
    std::vector<int> pos_of_orig(N, -1);
    for (int k = 0; k < M; k++) pos_of_orig[row_orig[k]] = k;
    std::vector<int> rows(M + 1, 0), cols;
    std::vector<std::vector<double>> vals(G);
    for (int k = 0; k < M; k++) {
        int r = row_orig[k];
        for (int q = sp.row_ptr[r]; q < sp.row_ptr[r + 1]; q++) {
            int c = sp.col[q];
            if (!reach[c]) continue;
            cols.push_back(pos_of_orig[c]);
            for (int g = 0; g < G; g++) vals[g].push_back(sp.val[(size_t)g * sp.nnz + q]);
        }
        rows[k + 1] = (int)cols.size();
    }
    const int nnz = (int)cols.size();
    std::vector<double> hv;
    for (int g = 0; g < G; g++) hv.insert(hv.end(), vals[g].begin(), vals[g].end());
    std::vector<double> rw(M, 0.0);
    if (h_rw)
        for (int k = 0; k < M; k++) rw[k] = h_rw[row_orig[k]];

    // ---- norm bound -> Taylor degree and sub-steps ----
    std::vector<double> h_prog((size_t)ntraj * nch * nseg * 5);
    SSS_CUDA(cudaMemcpyAsync(h_prog.data(), d_prog, sizeof(double) * h_prog.size(), cudaMemcpyDeviceToHost, st));
    SSS_CUDA(cudaStreamSynchronize(st));
    std::vector<double> cmax(G, 0.0);
    cmax[0] = 1.0;
    for (int b = 0; b < ntraj; b++)
        for (int c = 0; c < nch && c + 1 < G; c++)
            for (int s = 0; s < nseg; s++) {
                const double* q = &h_prog[(((size_t)b * nch + c) * nseg + s) * 5];
                cmax[c + 1] = std::max(cmax[c + 1], std::fabs(q[1]) + std::fabs(q[2]));
            }
    double wsum = 0.0;
    for (int e = 0; e < p->d.K; e++) {
        double s = 0.0;
        for (int k = 0; k < p->d.Q; k++) s += std::fabs(p->W[e * p->d.Q + k]);
        wsum = std::max(wsum, s);
    }
    double beta = 0.0;
    for (int g = 0; g < G; g++) {
        // 1-norm of the generator restricted to reachable rows/cols
        std::vector<double> colsum(M, 0.0);
        for (int k = 0; k < M; k++)
            for (int q = rows[k]; q < rows[k + 1]; q++) colsum[cols[q]] += std::fabs(vals[g][q - 0 * rows[0]]);
        double n1 = colsum.empty() ? 0.0 : *std::max_element(colsum.begin(), colsum.end());
        beta += cmax[g] * n1;
    }
    beta *= wsum * dt / F;
    int degree, substeps;
    choose_taylor(beta, p->d.taylor_degree, &degree, &substeps);

    // ---- upload the pattern ----
    std::vector<double> toff(F), noff(p->d.Q);
    for (int r = 0; r < F; r++) toff[r] = ((double)r * dt) / F;
    for (int k = 0; k < p->d.Q; k++) noff[k] = (dt * p->nodes[k]) / F;
    rw.insert(rw.end(), toff.begin(), toff.end());
    rw.insert(rw.end(), noff.begin(), noff.end());
    size_t words = hv.size() + rw.size();
    size_t ints = rows.size() + cols.size() + lane_rows.size() + row_orig.size();
    if (int rc = p->d_sp_val.ensure(sizeof(double) * words + sizeof(int) * ints + 64)) return rc;
    double* dv = p->d_sp_val.as<double>();
    int* di = reinterpret_cast<int*>(dv + words);
    std::vector<char> blob(sizeof(double) * words + sizeof(int) * ints);
    memcpy(blob.data(), hv.data(), sizeof(double) * hv.size());
    memcpy(blob.data() + sizeof(double) * hv.size(), rw.data(), sizeof(double) * rw.size());
    int* bi = reinterpret_cast<int*>(blob.data() + sizeof(double) * words);
    memcpy(bi, rows.data(), sizeof(int) * rows.size());
    memcpy(bi + rows.size(), cols.data(), sizeof(int) * cols.size());
    memcpy(bi + rows.size() + cols.size(), lane_rows.data(), sizeof(int) * lane_rows.size());
    memcpy(bi + rows.size() + cols.size() + lane_rows.size(), row_orig.data(), sizeof(int) * row_orig.size());
    SSS_CUDA(cudaMemcpyAsync(dv, blob.data(), blob.size(), cudaMemcpyHostToDevice, st));
    if (int rc = p->w_queue.ensure(sizeof(int) * 4)) return rc;
    SSS_CUDA(cudaMemsetAsync(p->w_queue.p, 0, sizeof(int) * 4, st));

    BatchArgs a{};
    a.M = M; a.G = G; a.K = p->d.K; a.Q = p->d.Q; a.F = F; a.nch = nch; a.nseg = nseg;
    a.T_max = T_max; a.ntraj = ntraj; a.degree = degree; a.substeps = substeps; a.nnz = nnz;
    a.h_sub = dt / F / substeps; a.t0 = t0; a.dt = dt;
    a.W = p->d_gens.as<double>() + p->gens.size();
    a.nodes = a.W + p->d.K * p->d.Q;
    a.vals = dv;
    a.rw = h_rw ? dv + hv.size() : nullptr;
    a.toff = dv + hv.size() + M;
    a.noff = a.toff + F;
    a.rows = di;
    a.cols = di + rows.size();
    a.lane_rows = di + rows.size() + cols.size();
    a.row_orig = di + rows.size() + cols.size() + lane_rows.size();
    a.rho0 = d_rho0; a.prog = d_prog; a.samples = d_samples; a.N = N;
    a.readout = d_readout; a.fin = d_final;
    a.queue = p->w_queue.as<int>();
    for (int j = 0; j <= kMaxTaylor; j++) a.inv_j[j] = j ? 1.0 / j : 0.0;

    const int threads = p->batch_threads > 0 ? p->batch_threads : 128;
    size_t shared_words = (size_t)G * nnz + M + ((M + 1 + nnz + L + 1 + 1) / 2);
    size_t per_slot = (size_t)nnz + 4 * M + kMaxQ * kMaxG;
    size_t smem = sizeof(double) * (shared_words + (threads / L) * per_slot);
    if (smem > 227 * 1024)
        return fail(SSS_EINVAL, "batched kernel needs " + std::to_string(smem) +
                                    " bytes of shared memory per CTA (max 232448); use more lanes per trajectory");
    int rc;
    switch (L) {
        case 1: rc = launch_batch<1>(p, a, threads, smem, st); break;
        case 2: rc = launch_batch<2>(p, a, threads, smem, st); break;
        case 4: rc = launch_batch<4>(p, a, threads, smem, st); break;
        case 8: rc = launch_batch<8>(p, a, threads, smem, st); break;
        case 16: rc = launch_batch<16>(p, a, threads, smem, st); break;
        default: rc = launch_batch<32>(p, a, threads, smem, st); break;
    }
    p->last_launches = rc == SSS_OK ? 1 : 0;
    p->last_batch_lanes = L;
    p->last_degree = degree;
    p->last_substeps = substeps;
    p->last_rows = M;
    p->last_nnz = nnz;
    return rc;
}

}  // namespace sss
