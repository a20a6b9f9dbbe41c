// C-ABI entry points of libsss.so (declared in include/sss.h): plan
// set-up (the reference's generate_simulator set-up,
// superspinsim/generate_simulator.py:49-154 and :1683-1814), argument
// checking, host<->device staging, and dispatch to the plain and batched
// paths.  No exception or abort crosses the ABI.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>

#include "sss_internal.cuh"

namespace sss {

static thread_local std::string g_error;

void set_error(const std::string& msg) { g_error = msg; }

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_error = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return SSS_ENOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return SSS_ENODEVICE;
    return SSS_ECUDA;
}

int DevBuf::ensure(size_t n) {
    if (n <= bytes && p) return SSS_OK;
    release();
    if (n == 0) return SSS_OK;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
        p = nullptr;
        bytes = 0;
        return cuda_fail(e, "cudaMalloc");
    }
    bytes = n;
    return SSS_OK;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

static int upload(DevBuf& buf, const double* h, size_t n) {
    if (int rc = buf.ensure(n * sizeof(double))) return rc;
    if (n) SSS_CUDA(cudaMemcpy(buf.p, h, n * sizeof(double), cudaMemcpyHostToDevice));
    return SSS_OK;
}

static bool finite_all(const double* a, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (!std::isfinite(a[i])) return false;
    return true;
}

}  // namespace sss

using namespace sss;

extern "C" {

const char* sss_last_error(void) { return g_error.c_str(); }

int sss_plan_create(sss_plan** out, const sss_plan_desc* d, const double* generators,
                    const double* weights, const double* nodes) {
    if (!out || !d) return fail(SSS_EINVAL, "null plan or descriptor");
    *out = nullptr;
    if (d->N <= 0 || d->G <= 0 || d->G > kMaxG || d->K <= 0 || d->K > kMaxK || d->Q <= 0 ||
        d->Q > kMaxQ)
        return fail(SSS_EINVAL, "bad plan shape (N, G, K, Q)");
    if (d->expm != SSS_EXPM_REFERENCE && d->expm != SSS_EXPM_TAYLOR)
        return fail(SSS_EINVAL, "unknown exponential algorithm");
    if (d->expm == SSS_EXPM_REFERENCE && (d->quartic_repeats < 0 || d->quartic_repeats > 500))
        return fail(SSS_EINVAL, "quartic_repeats out of range");
    if (!weights || !nodes) return fail(SSS_EINVAL, "null weights or nodes");
    bool rotating = (d->flags & SSS_ROTATING) != 0;
    if (!rotating && !generators) return fail(SSS_EINVAL, "null generators");
    int dev_count = 0;
    cudaError_t ce = cudaGetDeviceCount(&dev_count);
    if (ce != cudaSuccess || dev_count == 0)
        return fail(SSS_ENODEVICE, std::string("no CUDA device: ") + cudaGetErrorString(ce));
    sss_plan* p = new (std::nothrow) sss_plan();
    if (!p) return fail(SSS_ENOMEM, "host allocation failed");
    p->d = *d;
    p->rotating = rotating;
    memcpy(p->W, weights, sizeof(double) * d->K * d->Q);
    memcpy(p->nodes, nodes, sizeof(double) * d->Q);
    if (cudaGetDevice(&p->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess) {
        delete p;
        return fail(SSS_ECUDA, "cannot query the current device");
    }
    size_t NN = (size_t)d->N * d->N;
    if (!rotating) {
        p->gens.assign(generators, generators + (size_t)d->G * NN);
        if (!finite_all(p->gens.data(), p->gens.size())) {
            delete p;
            return fail(SSS_ENONFINITE, "generators contain NaN or Inf");
        }
        // device layout: generators, then W (K*Q), then nodes (Q)
        std::vector<double> packed(p->gens);
        packed.insert(packed.end(), p->W, p->W + d->K * d->Q);
        packed.insert(packed.end(), p->nodes, p->nodes + d->Q);
        if (int rc = upload(p->d_gens, packed.data(), packed.size())) {
            delete p;
            return rc;
        }
        if (int rc = build_sparse(p)) {
            sss_plan_destroy(p);
            return rc;
        }
    }
    *out = p;
    return SSS_OK;
}

int sss_plan_set_rotating(sss_plan* p, const double* gn, const double* dlast, int D,
                          const double* slast, int S, const double* V, const double* Vinv) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    if (!p->rotating) return fail(SSS_EINVAL, "plan was not created with SSS_ROTATING");
    const int N = p->d.N;
    if (D < 0 || S < 0 || 2 * D + S != N) return fail(SSS_EINVAL, "2D + S must equal N");
    if (!gn || !V || !Vinv || (D && !dlast) || (S && !slast))
        return fail(SSS_EINVAL, "null rotating-frame table");
    size_t NN = (size_t)N * N;
    p->gens.assign(gn, gn + (size_t)p->d.Q * p->d.G * NN);
    std::vector<double> packed(p->gens);
    packed.insert(packed.end(), p->W, p->W + p->d.K * p->d.Q);
    packed.insert(packed.end(), p->nodes, p->nodes + p->d.Q);
    if (int rc = upload(p->d_gens, packed.data(), packed.size())) return rc;
    p->D = D;
    p->S = S;
    p->dlast.assign(dlast, dlast + 2 * (size_t)D);
    p->slast.assign(slast, slast + (size_t)S);
    p->V.assign(V, V + NN);
    p->Vinv.assign(Vinv, Vinv + NN);
    if (int rc = upload(p->d_dlast, p->dlast.data(), p->dlast.size())) return rc;
    if (int rc = upload(p->d_slast, p->slast.data(), p->slast.size())) return rc;
    if (int rc = upload(p->d_V, V, NN)) return rc;
    if (int rc = upload(p->d_Vinv, Vinv, NN)) return rc;
    return build_sparse(p);  // (node, generator) slots for batched runs
}

int sss_plan_set_projection(sss_plan* p, int n_full, const double* P) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    if (p->u_n) return fail(SSS_EINVAL, "a unitary-mode plan cannot take a projection");
    if (n_full == 0) {
        p->n_full = 0;
        return SSS_OK;
    }
    const int N = p->d.N;
    if (n_full < N || !P) return fail(SSS_EINVAL, "projection needs n_full >= N and P (n_full x N)");
    if (!finite_all(P, (size_t)n_full * N)) return fail(SSS_ENONFINITE, "projection contains NaN or Inf");
    if (int rc = upload(p->d_P, P, (size_t)n_full * N)) return rc;
    p->n_full = n_full;
    return SSS_OK;
}

int sss_plan_set_unitary(sss_plan* p, int n, int nd, const int* map) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    if (p->n_full) return fail(SSS_EINVAL, "a projected plan cannot run in unitary mode");
    if (n == 0) {
        p->u_n = 0;
        return SSS_OK;
    }
    if (n < 1 || 2 * n != p->d.N) return fail(SSS_EINVAL, "unitary mode needs N = 2n");
    if (map) {
        if (nd < 1 || nd > 2 * n * n) return fail(SSS_EINVAL, "bad vectorisation map size");
        for (int i = 0; i < nd; i++) {
            const int y = map[3 * i], x = map[3 * i + 1], c = map[3 * i + 2];
            if (y < 0 || y >= n || x < 0 || x >= n || c < 0 || c > 1)
                return fail(SSS_EINVAL, "vectorisation map entry out of range");
        }
        std::vector<double> m(map, map + 3 * (size_t)nd);  // stored as doubles
        if (int rc = upload(p->d_umap, m.data(), m.size())) return rc;
    } else {
        nd = 2 * n * n;
    }
    p->u_n = n;
    p->u_nd = nd;
    p->u_mapped = map != nullptr;
    return SSS_OK;
}

static int check_run(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                     const double* programs, const double* tab, double dt, int T, int F,
                     const void* out) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    if (p->rotating && p->D + p->S == 0) return fail(SSS_EINVAL, "rotating tables not set");
    if (ntraj < 0 || T < 0 || F <= 0) return fail(SSS_EINVAL, "bad ntraj, T or F");
    if (ntraj == 0 || T == 0) return SSS_OK;
    if (!rho0 || !out) return fail(SSS_EINVAL, "null rho0 or output");
    if (!programs && !tab) return fail(SSS_EINVAL, "need a coefficient program or table");
    if (programs && (nch < 0 || nch > kMaxCh || nseg <= 0))
        return fail(SSS_EINVAL, "bad program shape");
    if (!(dt > 0) || !std::isfinite(dt)) return fail(SSS_EINVAL, "dt must be positive and finite");
    return SSS_OK;
}

static int simulate_impl(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                         const double* programs, const double* tab, double t0, double dt, int T,
                         int F, double* out, void* stream, bool host) {
    if (int rc = check_run(p, ntraj, rho0, nch, nseg, programs, tab, dt, T, F, out)) return rc;
    p->last_launches = 0;
    if (ntraj == 0 || T == 0) return SSS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int N = p->state_in();  // entries of a state in and of a sample out
    const double *d_rho0 = rho0, *d_prog = programs, *d_tab = tab;
    double* d_out = out;
    if (host) {
        size_t nprog = programs ? (size_t)ntraj * nch * nseg * 5 : 0;
        size_t ntab = tab ? (size_t)ntraj * F * T * p->d.Q * p->d.G : 0;
        if (programs && !finite_all(programs, nprog) ) {
            // +-inf segment ends are allowed; NaN is not
            for (size_t i = 0; i < nprog; i++)
                if (std::isnan(programs[i])) return fail(SSS_ENONFINITE, "program contains NaN");
        }
        if (int rc = p->w_in.ensure(sizeof(double) * ((size_t)ntraj * N + nprog + ntab))) return rc;
        if (int rc = p->w_out.ensure(sizeof(double) * (size_t)ntraj * T * N)) return rc;
        double* base = p->w_in.as<double>();
        SSS_CUDA(cudaMemcpyAsync(base, rho0, sizeof(double) * ntraj * N, cudaMemcpyHostToDevice, st));
        d_rho0 = base;
        if (programs) {
            SSS_CUDA(cudaMemcpyAsync(base + (size_t)ntraj * N, programs, sizeof(double) * nprog,
                                     cudaMemcpyHostToDevice, st));
            d_prog = base + (size_t)ntraj * N;
        }
        if (tab) {
            SSS_CUDA(cudaMemcpyAsync(base + (size_t)ntraj * N + nprog, tab, sizeof(double) * ntab,
                                     cudaMemcpyHostToDevice, st));
            d_tab = base + (size_t)ntraj * N + nprog;
        }
        d_out = p->w_out.as<double>();
    }
    int rc = plain_run(p, ntraj, d_rho0, nch, nseg, d_prog, d_tab, t0, dt, T, F, d_out, st);
    if (rc) return rc;
    if (host) {
        SSS_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * (size_t)ntraj * T * N,
                                 cudaMemcpyDeviceToHost, st));
        SSS_CUDA(cudaStreamSynchronize(st));
        for (size_t i = 0; i < (size_t)ntraj * T * N; i++)
            if (!std::isfinite(out[i])) return fail(SSS_ENONFINITE, "state became NaN or Inf");
    }
    return SSS_OK;
}

int sss_simulate(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                 const double* programs, const double* tab, double t0, double dt, int T, int F,
                 double* out, void* stream) {
    return simulate_impl(p, ntraj, rho0, nch, nseg, programs, tab, t0, dt, T, F, out, stream, true);
}

int sss_simulate_device(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                        const double* programs, const double* tab, double t0, double dt, int T,
                        int F, double* out, void* stream) {
    return simulate_impl(p, ntraj, rho0, nch, nseg, programs, tab, t0, dt, T, F, out, stream, false);
}

// sss_batch_run and sss_batch_run_table: programs, or a coefficient table
static int batch_run_impl(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                          const double* programs, const double* tab, const int* samples, double t0,
                          double dt, int T_max, int F, const double* readout_weights,
                          double* readout, double* final_state, double* trace, int host,
                          void* stream) {
    if (int rc = check_run(p, ntraj, rho0, nch, nseg, programs, tab, dt, T_max, F,
                           readout ? (const void*)readout
                                   : (final_state ? (const void*)final_state : (const void*)trace)))
        return rc;
    if (!programs && !tab)
        return fail(SSS_EINVAL, "batched runs need a coefficient program or table");
    if (tab) {
        nch = p->d.G;
        nseg = 0;
    }
    if (p->rotating && p->D + p->S == 0) return fail(SSS_EINVAL, "rotating tables not set");
    if (p->n_full || p->u_n)
        return fail(SSS_EINVAL, "batched runs support neither projected nor unitary plans");
    if (readout && !readout_weights) return fail(SSS_EINVAL, "readout needs readout_weights");
    p->last_launches = 0;
    if (ntraj == 0 || T_max == 0) return SSS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int N = p->d.N;
    // per-trajectory sample counts (host copy needed for the reachability
    // analysis and for validation)
    std::vector<int> h_samples;
    if (samples) {
        h_samples.resize(ntraj);
        if (host) {
            memcpy(h_samples.data(), samples, sizeof(int) * ntraj);
        } else {
            SSS_CUDA(cudaMemcpy(h_samples.data(), samples, sizeof(int) * ntraj, cudaMemcpyDeviceToHost));
        }
        for (int b = 0; b < ntraj; b++)
            if (h_samples[b] < 0 || h_samples[b] > T_max)
                return fail(SSS_EINVAL, "samples[b] must lie in [0, T_max]");
    }
    const double *d_rho0 = rho0, *d_prog = programs, *d_tab = tab;
    const int* d_samples = samples;
    double *d_ro = readout, *d_fin = final_state, *d_tr = trace;
    const size_t nprog = tab ? 0 : (size_t)ntraj * nch * nseg * 5;
    const size_t ntab = tab ? (size_t)ntraj * F * T_max * p->d.Q * p->d.G : 0;
    if (host) {
        for (size_t i = 0; i < nprog; i++)
            if (std::isnan(programs[i])) return fail(SSS_ENONFINITE, "program contains NaN");
        if (int rc = p->w_in.ensure(sizeof(double) * ((size_t)ntraj * N + nprog + ntab))) return rc;
        double* base = p->w_in.as<double>();
        SSS_CUDA(cudaMemcpyAsync(base, rho0, sizeof(double) * ntraj * N, cudaMemcpyHostToDevice, st));
        d_rho0 = base;
        if (tab) {
            SSS_CUDA(cudaMemcpyAsync(base + (size_t)ntraj * N, tab, sizeof(double) * ntab,
                                     cudaMemcpyHostToDevice, st));
            d_tab = base + (size_t)ntraj * N;
        } else {
            SSS_CUDA(cudaMemcpyAsync(base + (size_t)ntraj * N, programs, sizeof(double) * nprog,
                                     cudaMemcpyHostToDevice, st));
            d_prog = base + (size_t)ntraj * N;
        }
        if (samples) {
            if (int rc = p->w_samples.ensure(sizeof(int) * ntraj)) return rc;
            SSS_CUDA(cudaMemcpyAsync(p->w_samples.p, samples, sizeof(int) * ntraj,
                                     cudaMemcpyHostToDevice, st));
            d_samples = p->w_samples.as<int>();
        }
        if (readout) {
            if (int rc = p->w_ro.ensure(sizeof(double) * (size_t)ntraj * T_max)) return rc;
            d_ro = p->w_ro.as<double>();
        }
        if (final_state) {
            if (int rc = p->w_fin.ensure(sizeof(double) * (size_t)ntraj * N)) return rc;
            d_fin = p->w_fin.as<double>();
        }
        if (trace) {
            if (int rc = p->w_out.ensure(sizeof(double) * (size_t)ntraj * T_max * N)) return rc;
            d_tr = p->w_out.as<double>();
        }
    }
    int rc = batch_run(p, ntraj, d_rho0, nch, nseg, tab ? nullptr : d_prog, d_samples,
                       samples ? h_samples.data() : nullptr, t0, dt, T_max, F, readout_weights,
                       d_ro, d_fin, st, d_tr, d_tab);
    if (rc) return rc;
    if (host) {
        if (readout)
            SSS_CUDA(cudaMemcpyAsync(readout, d_ro, sizeof(double) * (size_t)ntraj * T_max,
                                     cudaMemcpyDeviceToHost, st));
        if (final_state)
            SSS_CUDA(cudaMemcpyAsync(final_state, d_fin, sizeof(double) * (size_t)ntraj * N,
                                     cudaMemcpyDeviceToHost, st));
        if (trace)
            SSS_CUDA(cudaMemcpyAsync(trace, d_tr, sizeof(double) * (size_t)ntraj * T_max * N,
                                     cudaMemcpyDeviceToHost, st));
        SSS_CUDA(cudaStreamSynchronize(st));
        return batch_check(p, st);
    }
    return SSS_OK;
}

int sss_batch_run(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                  const double* programs, const int* samples, double t0, double dt, int T_max,
                  int F, const double* readout_weights, double* readout, double* final_state,
                  double* trace, int host, void* stream) {
    return batch_run_impl(p, ntraj, rho0, nch, nseg, programs, nullptr, samples, t0, dt, T_max, F,
                          readout_weights, readout, final_state, trace, host, stream);
}

int sss_batch_run_table(sss_plan* p, int ntraj, const double* rho0, const double* coeff_table,
                        const int* samples, double t0, double dt, int T_max, int F,
                        const double* readout_weights, double* readout, double* final_state,
                        double* trace, int host, void* stream) {
    return batch_run_impl(p, ntraj, rho0, 0, 0, nullptr, coeff_table, samples, t0, dt, T_max, F,
                          readout_weights, readout, final_state, trace, host, stream);
}

static int adjoint_impl(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                        const double* programs, double t0, double dt, int T, int F,
                        const double* readout_weights, const double* time_weights, int channel,
                        int npar, double* J, double* grad, int host, void* stream) {
    if (int rc = check_run(p, ntraj, rho0, nch, nseg, programs, nullptr, dt, T, F,
                           (const void*)J))
        return rc;
    if (!programs || !readout_weights || !time_weights || !grad)
        return fail(SSS_EINVAL, "the adjoint needs programs, readout and time weights, and grad");
    if (p->rotating) return fail(SSS_EINVAL, "the adjoint supports the lab frame only");
    if (p->n_full || p->u_n)
        return fail(SSS_EINVAL, "the adjoint supports neither projected nor unitary plans");
    p->last_launches = 0;
    if (ntraj == 0 || T == 0) return SSS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int N = p->d.N;
    const double *d_rho0 = rho0, *d_prog = programs;
    double *d_J = J, *d_grad = grad;
    size_t nprog = (size_t)ntraj * nch * nseg * 5;
    if (host) {
        for (size_t i = 0; i < nprog; i++)
            if (std::isnan(programs[i])) return fail(SSS_ENONFINITE, "program contains NaN");
        if (int rc = p->w_in.ensure(sizeof(double) * ((size_t)ntraj * N + nprog))) return rc;
        if (int rc = p->w_out.ensure(sizeof(double) * ((size_t)ntraj + (size_t)ntraj * nseg * npar)))
            return rc;
        double* base = p->w_in.as<double>();
        SSS_CUDA(cudaMemcpyAsync(base, rho0, sizeof(double) * ntraj * N, cudaMemcpyHostToDevice, st));
        SSS_CUDA(cudaMemcpyAsync(base + (size_t)ntraj * N, programs, sizeof(double) * nprog,
                                 cudaMemcpyHostToDevice, st));
        d_rho0 = base;
        d_prog = base + (size_t)ntraj * N;
        d_J = p->w_out.as<double>();
        d_grad = d_J + ntraj;
    }
    if (int rc = adjoint_run(p, ntraj, d_rho0, nch, nseg, d_prog, t0, dt, T, F, readout_weights,
                             time_weights, channel, npar, d_J, d_grad, st))
        return rc;
    if (host) {
        const size_t ng = (size_t)ntraj * nseg * npar;
        SSS_CUDA(cudaMemcpyAsync(J, d_J, sizeof(double) * ntraj, cudaMemcpyDeviceToHost, st));
        SSS_CUDA(cudaMemcpyAsync(grad, d_grad, sizeof(double) * ng, cudaMemcpyDeviceToHost, st));
        SSS_CUDA(cudaStreamSynchronize(st));
        if (!finite_all(J, (size_t)ntraj) || !finite_all(grad, ng))
            return fail(SSS_ENONFINITE, "adjoint objective or gradient became NaN or Inf");
    }
    return SSS_OK;
}

int sss_adjoint_run(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                    const double* programs, double t0, double dt, int T, int F,
                    const double* readout_weights, const double* time_weights, double* J,
                    double* grad, int host, void* stream) {
    return adjoint_impl(p, ntraj, rho0, nch, nseg, programs, t0, dt, T, F, readout_weights,
                        time_weights, 0, 2, J, grad, host, stream);
}

int sss_adjoint_run_channel(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                            const double* programs, double t0, double dt, int T, int F,
                            const double* readout_weights, const double* time_weights,
                            int channel, double* J, double* grad, int host, void* stream) {
    return adjoint_impl(p, ntraj, rho0, nch, nseg, programs, t0, dt, T, F, readout_weights,
                        time_weights, channel, 4, J, grad, host, stream);
}

int sss_batch_prepare(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                      const double* programs, double dt, int F, const double* readout_weights,
                      void* stream) {
    if (int rc = check_run(p, ntraj, rho0, nch, nseg, programs, nullptr, dt, 1, F, rho0)) return rc;
    if (!programs) return fail(SSS_EINVAL, "batched runs need a coefficient program");
    if (p->rotating && p->D + p->S == 0) return fail(SSS_EINVAL, "rotating tables not set");
    if (p->n_full || p->u_n)
        return fail(SSS_EINVAL, "batched runs support neither projected nor unitary plans");
    if (ntraj == 0) return fail(SSS_EINVAL, "empty batch");
    return batch_prepare(p, ntraj, rho0, nch, nseg, programs, dt, F, readout_weights,
                         (cudaStream_t)stream);
}

int sss_batch_prepare_samples(sss_plan* p, int ntraj, const double* rho0, int nch, int nseg,
                              const double* programs, const int* samples, double dt, int F,
                              const double* readout_weights, void* stream) {
    if (int rc = check_run(p, ntraj, rho0, nch, nseg, programs, nullptr, dt, 1, F, rho0)) return rc;
    if (!programs) return fail(SSS_EINVAL, "batched runs need a coefficient program");
    if (!samples) return fail(SSS_EINVAL, "null samples");
    if (p->rotating && p->D + p->S == 0) return fail(SSS_EINVAL, "rotating tables not set");
    if (p->n_full || p->u_n)
        return fail(SSS_EINVAL, "batched runs support neither projected nor unitary plans");
    if (ntraj == 0) return fail(SSS_EINVAL, "empty batch");
    for (int b = 0; b < ntraj; b++)
        if (samples[b] < 0) return fail(SSS_EINVAL, "samples[b] must not be negative");
    return batch_prepare(p, ntraj, rho0, nch, nseg, programs, dt, F, readout_weights,
                         (cudaStream_t)stream, nullptr, 0, samples);
}

int sss_batch_launch(sss_plan* p, double* state, const double* programs, const int* samples,
                     double t0, int t_begin, int n_samples, int T_max, double* readout,
                     void* stream) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    if (!p->batch_ready) return fail(SSS_EINVAL, "no prepared batch (call sss_batch_prepare)");
    if (!state || !programs) return fail(SSS_EINVAL, "null state or programs");
    if (t_begin < 0 || n_samples < 0 || t_begin + n_samples > T_max)
        return fail(SSS_EINVAL, "need 0 <= t_begin and t_begin + n_samples <= T_max");
    return batch_launch(p, state, programs, samples, t0, t_begin, n_samples, T_max, readout,
                        (cudaStream_t)stream);
}

int sss_batch_check(sss_plan* p, void* stream) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    return batch_check(p, (cudaStream_t)stream);
}

int sss_plan_last_launches(const sss_plan* p) { return p ? p->last_launches : 0; }

int sss_slot_layout(int M, const int* row_ptr, const int* col, int lanes, int max_slots,
                    int* slots, int* barrier_slot, int* partials, unsigned* words, int* entries) {
    return sss::slot_layout_host(M, row_ptr, col, lanes, max_slots, slots, barrier_slot, partials,
                                 words, entries);
}

// FP64 FMA throughput probe: every thread runs 8 independent DFMA chains.
static __global__ void k_dfma_peak(double* out, int iters, double a, double b) {
    double x[8];
    for (int j = 0; j < 8; j++) x[j] = threadIdx.x * 1e-9 + j;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = fma(x[j], a, b);
    }
    double s = 0;
    for (int j = 0; j < 8; j++) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int sss_fp64_peak(double* tflops, void* stream) {
    if (!tflops) return fail(SSS_EINVAL, "null output");
    int dev = 0, sms = 0;
    SSS_CUDA(cudaGetDevice(&dev));
    SSS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = sms * 4, threads = 256, iters = 8192;
    double* buf = nullptr;
    SSS_CUDA(cudaMalloc(&buf, sizeof(double) * blocks * threads));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_dfma_peak<<<blocks, threads, 0, st>>>(buf, 256, 0.9999999, 1e-7);
    cudaEventRecord(e0, st);
    k_dfma_peak<<<blocks, threads, 0, st>>>(buf, iters, 0.9999999, 1e-7);
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, "fp64 peak probe");
    *tflops = 2.0 * 8 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    return SSS_OK;
}

// FP64 tensor-core (DMMA) throughput probe: mma.sync m8n8k4 f64 on 8
// independent accumulator tiles per warp in a bounded loop.
static __global__ void k_dmma_peak(double* out, int iters, double a, double b) {
    double c[8][2];
    for (int j = 0; j < 8; j++) {
        c[j][0] = 0.0;
        c[j][1] = 0.0;
    }
    const double x = a + threadIdx.x * 1e-12, y = b;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++)
            asm volatile(
                "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                : "+d"(c[j][0]), "+d"(c[j][1])
                : "d"(x), "d"(y));
    }
    double s = 0.0;
    for (int j = 0; j < 8; j++) s += c[j][0] + c[j][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int sss_fp64_mma_peak(double* tflops, void* stream) {
    if (!tflops) return fail(SSS_EINVAL, "null output");
    int dev = 0, sms = 0;
    SSS_CUDA(cudaGetDevice(&dev));
    SSS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = sms * 4, threads = 256, iters = 4096;
    double* buf = nullptr;
    SSS_CUDA(cudaMalloc(&buf, sizeof(double) * blocks * threads));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_dmma_peak<<<blocks, threads, 0, st>>>(buf, 128, 1e-3, 1e-3);
    cudaEventRecord(e0, st);
    k_dmma_peak<<<blocks, threads, 0, st>>>(buf, iters, 1e-3, 1e-3);
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, "fp64 tensor-core peak probe");
    // 2*8*8*4 flop per warp-wide m8n8k4, 8 tiles per iteration
    *tflops = 512.0 * 8 * iters * ((double)blocks * threads / 32) / (ms * 1e-3) / 1e12;
    return SSS_OK;
}

int sss_plan_set_batch_config(sss_plan* p, int lanes, int cta_threads, int variant) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    if (lanes < 0 || lanes > 256 || (lanes & (lanes - 1)))
        return fail(SSS_EINVAL, "lanes must be 0 (automatic) or a power of two up to 256");
    if (lanes > 32 && variant != 0 && variant != 4 && variant != 6)
        return fail(SSS_EINVAL, "more than 32 lanes per trajectory needs the row-part or "
                                "slot-packed variant");
    if (cta_threads != 0 && (cta_threads < 32 || cta_threads > 256 || cta_threads % 32))
        return fail(SSS_EINVAL, "cta_threads must be 0 or a multiple of 32 in [32, 256]");
    if (variant < 0 || variant > 7) return fail(SSS_EINVAL, "variant must be 0 to 7");
    p->batch_lanes = lanes;
    p->batch_threads = cta_threads;
    p->batch_variant = variant;
    return SSS_OK;
}

int sss_plan_set_adjoint_memory(sss_plan* p, size_t max_bytes) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    p->adj_max_bytes = max_bytes;
    return SSS_OK;
}

int sss_plan_batch_work(const sss_plan* p, int* variant, int* live_generators, int* live_nnz,
                        int* fp64_per_term) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    if (variant) *variant = p->last_variant;
    if (live_generators) *live_generators = p->last_n_live;
    if (live_nnz) *live_nnz = p->last_live_nnz;
    if (fp64_per_term) *fp64_per_term = p->last_fp64_per_term;
    return SSS_OK;
}

int sss_plan_bank_conflicts(const sss_plan* p, int* before, int* after) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    if (before) *before = p->last_bank_before;
    if (after) *after = p->last_bank_after;
    return SSS_OK;
}

int sss_plan_batch_info(const sss_plan* p, int* lanes, int* degree, int* substeps, int* rows,
                        int* nnz, double* kernel_ms) {
    if (!p) return fail(SSS_EINVAL, "null plan");
    if (kernel_ms) {
        *kernel_ms = 0.0;
        if (p->ev_recorded) {
            float ms = 0.f;
            SSS_CUDA(cudaEventSynchronize(p->ev_end));
            SSS_CUDA(cudaEventElapsedTime(&ms, p->ev_begin, p->ev_end));
            *kernel_ms = ms;
        }
    }
    if (lanes) *lanes = p->last_batch_lanes;
    if (degree) *degree = p->last_degree;
    if (substeps) *substeps = p->last_substeps;
    if (rows) *rows = p->last_rows;
    if (nnz) *nnz = p->last_nnz;
    return SSS_OK;
}

void sss_plan_destroy(sss_plan* p) {
    if (!p) return;
    DevBuf* bufs[] = {&p->d_gens, &p->d_dlast, &p->d_slast, &p->d_V, &p->d_Vinv,
                      &p->d_sp_rowptr, &p->d_sp_col, &p->d_row_map,
                      &p->w_prop, &p->w_in, &p->w_out, &p->w_prog, &p->w_tab, &p->w_aux,
                      &p->w_queue, &p->w_ro, &p->w_fin, &p->w_samples, &p->w_status,
                      &p->w_state, &p->w_adjf, &p->w_adjb, &p->w_states, &p->w_adjro,
                      &p->w_adjst, &p->w_order, &p->w_health};
    for (DevBuf* b : bufs) b->release();
    for (DevBuf& b : p->batch_tables) b.release();
    if (p->ev_begin) cudaEventDestroy(p->ev_begin);
    if (p->ev_end) cudaEventDestroy(p->ev_end);
    delete p;
}

}  // extern "C"
