/*
 * sss_oracle.c -- CPU oracle for the time-stepping hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load this library: to check the
 * CUDA path's results, or as the timed CPU baseline.  The product (superspinsim_gb300)
 * never calls it.
 *
 * It restates the CPU path of the reference's compiled simulator,
 * monashNV/superspinsim 1.3.2 `superspinsim/generate_simulator.py`
 * (`simulate`, :1508-2200), in plain C with OpenMP.  Two modes:
 *
 *   SSS_ORACLE_REFERENCE  the reference's own algorithm, loop for loop:
 *       time grid (:158-167), sampling (:235-271), coefficient weighting
 *       (:278-350), exponent assembly (:354-448, rotating :450-532),
 *       scaling by 4^-R (:534-578), 2R squarings in residual or plain
 *       arithmetic (:706-724, :882-897), product of the K exponentials into
 *       the step propagator (:726-798, :1259-1294), rotating-frame step
 *       (:901-1021), serial chain of the step propagators (:1204-1224,
 *       :1308-1321), frame sandwich (:1023-1171) and application to rho0
 *       (:1325-1390).  Sums run in the reference's order with separate
 *       multiply and add (build with -ffp-contract=off), so on the same
 *       inputs it agrees with the reference's CPU path run as plain Python.
 *
 *   SSS_ORACLE_VECTOR  the same integrator applied to the state vector one
 *       step at a time: each exponential acts on rho through its Taylor
 *       series of a given degree.  O(N^2) per term instead of O(N^3) per
 *       squaring; used for long windows after it has been checked against
 *       the reference mode on short ones.
 *
 * Coefficients come from a segment program evaluated with libm cos (the
 * same function the reference's samplers call through math.cos).
 *
 * Parity pinned: the .npz fixtures under tests/golden hold outputs of the reference itself.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SSS_ORACLE_REFERENCE 0
#define SSS_ORACLE_VECTOR 1

/* Coefficient channel program: nch channels x nseg segments x 5 doubles
 * (t_end, offset, amplitude, frequency, phase).  Channel value at time t is
 * offset + amplitude*cos(tau*frequency*t + phase) of the first segment with
 * t < t_end, else 0. */
static double channel_value(const double* prog, int nseg, int ch, double t) {
    const double tau = 6.283185307179586;
    for (int s = 0; s < nseg; s++) {
        const double* p = prog + ((size_t)ch * nseg + s) * 5;
        if (t < p[0]) {
            return p[1] + p[2] * cos(tau * p[3] * t + p[4]);
        }
    }
    return 0.0;
}

/* Sampler of the reference's front end (generate_generators.py:2317-2358):
 * lab frame writes [1, x, y, z, r]; rotating frame writes [x, y, z, r]. */
static void sample_row(const double* prog, int nseg, int nch, int lab,
                       double t, double* row, int G) {
    for (int g = 0; g < G; g++) row[g] = 0.0;
    if (lab) {
        row[0] = 1.0;
        for (int c = 0; c < nch && c + 1 < G; c++)
            row[c + 1] = channel_value(prog, nseg, c, t);
    } else {
        for (int c = 0; c < nch && c < G; c++)
            row[c] = channel_value(prog, nseg, c, t);
    }
}

typedef struct {
    int N, G, K, Q;
    const double* gens;    /* lab: G*N*N; rotating: Q*G*N*N */
    const double* W;       /* K*Q */
    const double* nodes;   /* Q */
    int rotating;
    const double* dfwd;    /* D*2: residual-aware e^{L0 h} 2x2 blocks */
    int D;
    const double* sfwd;    /* S */
    int S;
    const double* V;       /* N*N */
    const double* Vinv;    /* N*N */
    int residual;
    int R;                 /* quartic repeats: 2R squarings */
    int degree;            /* vector mode Taylor degree */
    const double* prog;
    int nch, nseg;
} oracle_desc;

/* ---- dense helpers, in the reference's loop order ---------------------- */

/* Column-major copy of a right operand, so the inner products below read
 * both operands contiguously.  The products and their summation order are
 * unchanged (k ascending), so results are bit for bit those of the
 * row-major loops. */
static double* transposed(const double* m, int N) {
    double* t = (double*)malloc((size_t)N * N * sizeof(double));
    if (!t) return NULL;
    for (int k = 0; k < N; k++)
        for (int x = 0; x < N; x++) t[(size_t)x * N + k] = m[(size_t)k * N + x];
    return t;
}

/* out = (res ? 2*in : 0) + in@in   (generate_simulator.py:706-724).
 * Returns -1 if the scratch copy cannot be allocated. */
static int square_mat(const double* in, double* out, int N, int res) {
    double* it = transposed(in, N);
    if (!it) return -1;
    for (int y = 0; y < N; y++)
        for (int x = 0; x < N; x++) {
            const double* a = in + (size_t)y * N;
            const double* b = it + (size_t)x * N;
            double acc = res ? 2 * in[y * N + x] : 0.0;
            for (int k = 0; k < N; k++) acc += a[k] * b[k];
            out[y * N + x] = acc;
        }
    free(it);
    return 0;
}

/* out = (res ? L + R : 0) + L@R   (generate_simulator.py:726-743) */
static int mul_mat(const double* L, const double* Rm, double* out, int N,
                   int res) {
    double* rt = transposed(Rm, N);
    if (!rt) return -1;
    for (int y = 0; y < N; y++)
        for (int x = 0; x < N; x++) {
            const double* a = L + (size_t)y * N;
            const double* b = rt + (size_t)x * N;
            double acc = res ? L[y * N + x] + Rm[y * N + x] : 0.0;
            for (int k = 0; k < N; k++) acc += a[k] * b[k];
            out[y * N + x] = acc;
        }
    free(rt);
    return 0;
}

/* Rotating-frame step, TE <- e^{L0 h} TE, residual aware
 * (generate_simulator.py:901-964; the single-block loop runs over the
 * singles, as in the reference's GPU kernel :955-964). */
static void apply_eig(const oracle_desc* d, const double* in, double* out) {
    int N = d->N;
    for (int y = 0; y < d->D; y++) {
        double a = d->dfwd[2 * y], b = d->dfwd[2 * y + 1];
        for (int x = 0; x < N; x++) {
            double re, im;
            if (d->residual) {
                re = (1 + a) * in[(2 * y) * N + x] - b * in[(2 * y + 1) * N + x];
                im = b * in[(2 * y) * N + x] + (1 + a) * in[(2 * y + 1) * N + x];
                if (x == 2 * y) { re += a; im += b; }
                if (x == 2 * y + 1) { re -= b; im += a; }
            } else {
                re = a * in[(2 * y) * N + x] - b * in[(2 * y + 1) * N + x];
                im = b * in[(2 * y) * N + x] + a * in[(2 * y + 1) * N + x];
            }
            out[(2 * y) * N + x] = re;
            out[(2 * y + 1) * N + x] = im;
        }
    }
    int off = 2 * d->D;
    for (int y = 0; y < d->S; y++) {
        double s = d->sfwd[y];
        for (int x = 0; x < N; x++) {
            double v;
            if (d->residual) {
                v = (1 + s) * in[(off + y) * N + x];
                if (y + off == x) v += s;
            } else {
                v = s * in[(off + y) * N + x];
            }
            out[(off + y) * N + x] = v;
        }
    }
}

/* Exponent for step sample t, exponential e: Omega = h*sum(...)
 * lab (:354-448):   wc[g] = sum_k W[e,k] c[k,g];  Om = h*sum_g wc[g]*Gen[g]
 * rotating (:450-532): Om = sum_k sum_g (Gen[k,g]*c[k,g]) * (h*W[e,k]) */
static void build_exponent(const oracle_desc* d, const double* coef /*Q*G*/,
                           int e, double h, double* Om) {
    int N = d->N, G = d->G, Q = d->Q;
    if (!d->rotating) {
        double wc[16];
        for (int g = 0; g < G; g++) {
            double acc = 0;
            for (int k = 0; k < Q; k++) acc += d->W[e * Q + k] * coef[k * G + g];
            wc[g] = acc;
        }
        for (int y = 0; y < N; y++)
            for (int x = 0; x < N; x++) {
                double acc = 0.0;
                for (int g = 0; g < G; g++)
                    acc += wc[g] * d->gens[((size_t)g * N + y) * N + x];
                Om[y * N + x] = h * acc;
            }
    } else {
        for (int y = 0; y < N; y++)
            for (int x = 0; x < N; x++) {
                double acc = 0;
                for (int k = 0; k < Q; k++)
                    for (int g = 0; g < G; g++) {
                        double m0 = d->gens[(((size_t)k * G + g) * N + y) * N + x] *
                                    coef[k * G + g];
                        double m1 = h * d->W[e * Q + k];
                        acc += m0 * m1;
                    }
                Om[y * N + x] = acc;
            }
    }
}

/* ---- reference mode ----------------------------------------------------- */

static int run_reference(const oracle_desc* d, double t0, double dt, int T,
                         int F, const double* rho0, double* out) {
    int N = d->N, G = d->G, K = d->K, Q = d->Q;
    size_t NN = (size_t)N * N;
    double* TE = (double*)calloc((size_t)T * NN, sizeof(double));
    if (!TE) return -1;
    double scale = pow(4.0, d->R);
    int bad = 0;

    for (int t = 0; t < T; t++)
        if (!d->residual)
            for (int i = 0; i < N; i++) TE[t * NN + i * N + i] = 1.0;

    for (int r = 0; r < F; r++) {
        double toff = r * dt / F;
        double tstart = t0 + toff;
#pragma omp parallel
        {
            double* Om = (double*)malloc(K * NN * sizeof(double));
            double* sc = (double*)malloc(NN * sizeof(double));
            double* sc2 = (double*)malloc(NN * sizeof(double));
            double coef[64];
            if (!Om || !sc || !sc2) {
#pragma omp atomic write
                bad = 1;
            } else {
#pragma omp for schedule(static)
                for (int t = 0; t < T; t++) {
                    double tbase = tstart + dt * t;
                    for (int k = 0; k < Q; k++) {
                        double tn = tbase + dt * d->nodes[k] / F;
                        sample_row(d->prog, d->nseg, d->nch, !d->rotating, tn,
                                   coef + k * G, G);
                    }
                    for (int e = 0; e < K; e++) {
                        double* O = Om + e * NN;
                        build_exponent(d, coef, e, dt / F, O);
                        for (size_t i = 0; i < NN; i++) {
                            O[i] /= scale;
                        }
                        if (!d->residual)
                            for (int i = 0; i < N; i++) O[i * N + i] += 1.0;
                        for (int q = 0; q < d->R; q++) {
                            if (square_mat(O, sc, N, d->residual) ||
                                square_mat(sc, O, N, d->residual)) {
#pragma omp atomic write
                                bad = 1;
                            }
                        }
                    }
                    double* te = TE + t * NN;
                    /* :1259-1294 -- exponential K-1 first, 0 last */
                    for (int e = 0; e < K; e += 2) {
                        int rc = mul_mat(Om + (K - e - 1) * NN, te, sc, N, d->residual);
                        if (e + 1 < K)
                            rc |= mul_mat(Om + (K - e - 2) * NN, sc, te, N, d->residual);
                        else
                            memcpy(te, sc, NN * sizeof(double));
                        if (rc) {
#pragma omp atomic write
                            bad = 1;
                        }
                    }
                    if (d->rotating) {
                        apply_eig(d, te, sc2);
                        memcpy(te, sc2, NN * sizeof(double));
                    }
                }
            }
            free(Om);
            free(sc);
            free(sc2);
        }
        if (bad) {
            free(TE);
            return -1;
        }
    }
    /* serial chain :1308-1321 */
    double* sc = (double*)malloc(NN * sizeof(double));
    if (!sc) { free(TE); return -1; }
    for (int t = 0; t + 1 < T; t++) {
        if (mul_mat(TE + (t + 1) * NN, TE + t * NN, sc, N, d->residual)) {
            free(sc);
            free(TE);
            return -1;
        }
        memcpy(TE + (t + 1) * NN, sc, NN * sizeof(double));
    }
    free(sc);
    if (d->rotating) {
        /* :1023-1063 sandwich, V (I+TE) Vinv - I in residual form */
#pragma omp parallel
        {
            double* a = (double*)malloc(NN * sizeof(double));
#pragma omp for schedule(static)
            for (int t = 0; t < T; t++) {
                double* te = TE + t * NN;
                for (int y = 0; y < N; y++)
                    for (int x = 0; x < N; x++) {
                        double acc = d->residual ? d->Vinv[y * N + x] - (y == x) : 0.0;
                        for (int k = 0; k < N; k++) acc += te[y * N + k] * d->Vinv[k * N + x];
                        a[y * N + x] = acc;
                    }
                for (int y = 0; y < N; y++)
                    for (int x = 0; x < N; x++) {
                        double acc = d->residual ? d->V[y * N + x] - (y == x) : 0.0;
                        for (int k = 0; k < N; k++) acc += d->V[y * N + k] * a[k * N + x];
                        te[y * N + x] = acc;
                    }
            }
            free(a);
        }
    }
    /* :1325-1390 */
    for (int t = 0; t < T; t++)
        for (int i = 0; i < N; i++) {
            double acc = d->residual ? rho0[i] : 0.0;
            for (int k = 0; k < N; k++) acc += TE[t * NN + i * N + k] * rho0[k];
            out[(size_t)t * N + i] = acc;
        }
    free(TE);
    return 0;
}

/* ---- vector mode -------------------------------------------------------- */

/* The exponent on the union pattern of the generators (entries that are
 * zero in every generator are zero in every exponent): row_ptr (N+1) and
 * col (nnz, increasing within a row).  Skipping exact zeros leaves every
 * sum of the dense forms unchanged (up to the sign of a zero result). */
typedef struct {
    int nnz;
    int* row_ptr;
    int* col;
} oracle_pattern;

static int build_pattern(const oracle_desc* d, oracle_pattern* pt) {
    int N = d->N, planes = d->rotating ? d->Q * d->G : d->G;
    pt->row_ptr = (int*)malloc((size_t)(N + 1) * sizeof(int));
    pt->col = (int*)malloc((size_t)N * N * sizeof(int));
    if (!pt->row_ptr || !pt->col) return -1;
    int nnz = 0;
    for (int y = 0; y < N; y++) {
        pt->row_ptr[y] = nnz;
        for (int x = 0; x < N; x++) {
            int any = 0;
            for (int g = 0; g < planes && !any; g++)
                any = d->gens[((size_t)g * N + y) * N + x] != 0.0;
            if (any) pt->col[nnz++] = x;
        }
    }
    pt->row_ptr[N] = nnz;
    pt->nnz = nnz;
    return 0;
}

/* build_exponent restricted to the pattern: val[p] = Omega[y][col[p]],
 * formed with the same operations in the same order */
static void build_exponent_sparse(const oracle_desc* d, const oracle_pattern* pt,
                                  const double* coef, int e, double h, double* val) {
    int N = d->N, G = d->G, Q = d->Q;
    if (!d->rotating) {
        double wc[16];
        for (int g = 0; g < G; g++) {
            double acc = 0;
            for (int k = 0; k < Q; k++) acc += d->W[e * Q + k] * coef[k * G + g];
            wc[g] = acc;
        }
        for (int y = 0; y < N; y++)
            for (int p = pt->row_ptr[y]; p < pt->row_ptr[y + 1]; p++) {
                int x = pt->col[p];
                double acc = 0.0;
                for (int g = 0; g < G; g++)
                    acc += wc[g] * d->gens[((size_t)g * N + y) * N + x];
                val[p] = h * acc;
            }
    } else {
        for (int y = 0; y < N; y++)
            for (int p = pt->row_ptr[y]; p < pt->row_ptr[y + 1]; p++) {
                int x = pt->col[p];
                double acc = 0;
                for (int k = 0; k < Q; k++)
                    for (int g = 0; g < G; g++) {
                        double m0 = d->gens[(((size_t)k * G + g) * N + y) * N + x] *
                                    coef[k * G + g];
                        double m1 = h * d->W[e * Q + k];
                        acc += m0 * m1;
                    }
                val[p] = acc;
            }
    }
}

/* v <- exp(Om) v by Taylor series of the given degree (residual form:
 * the increment sum_{j>=1} Om^j v / j! is added to v at the end); Om on
 * the pattern. */
static void expv(const oracle_pattern* pt, const double* val, double* v, int N, int degree,
                 double* term, double* next, double* incr) {
    memcpy(term, v, N * sizeof(double));
    for (int i = 0; i < N; i++) incr[i] = 0.0;
    for (int j = 1; j <= degree; j++) {
        for (int y = 0; y < N; y++) {
            double acc = 0.0;
            for (int p = pt->row_ptr[y]; p < pt->row_ptr[y + 1]; p++)
                acc += val[p] * term[pt->col[p]];
            next[y] = acc / j;
        }
        for (int i = 0; i < N; i++) incr[i] += next[i];
        double* tmp = term;
        term = next;
        next = tmp;
    }
    for (int i = 0; i < N; i++) v[i] += incr[i];
}

static int run_vector(const oracle_desc* d, double t0, double dt, int T,
                      int F, const double* rho0, double* out) {
    int N = d->N, G = d->G, K = d->K, Q = d->Q;
    size_t NN = (size_t)N * N;
    oracle_pattern pt = {0, NULL, NULL};
    double* Om = (double*)malloc(NN * sizeof(double));
    double* v = (double*)malloc(5 * N * sizeof(double));
    if (!Om || !v || build_pattern(d, &pt)) {
        free(Om); free(v); free(pt.row_ptr); free(pt.col);
        return -1;
    }
    double *term = v + N, *next = v + 2 * N, *incr = v + 3 * N, *tmp = v + 4 * N;
    double coef[64];
    memcpy(v, rho0, N * sizeof(double));
    double h = dt / F;
    for (int t = 0; t < T; t++) {
        for (int r = 0; r < F; r++) {
            double tbase = (t0 + r * dt / F) + dt * t;
            for (int k = 0; k < Q; k++) {
                double tn = tbase + dt * d->nodes[k] / F;
                sample_row(d->prog, d->nseg, d->nch, !d->rotating, tn, coef + k * G, G);
            }
            for (int e = K - 1; e >= 0; e--) {
                build_exponent_sparse(d, &pt, coef, e, h, Om);
                expv(&pt, Om, v, N, d->degree, term, next, incr);
            }
            if (d->rotating) {
                /* v <- e^{L0 h} v with the residual-aware blocks */
                for (int y = 0; y < d->D; y++) {
                    double a = d->dfwd[2 * y], b = d->dfwd[2 * y + 1];
                    double re = v[2 * y], im = v[2 * y + 1];
                    if (d->residual) {
                        tmp[2 * y] = re + (a * re - b * im);
                        tmp[2 * y + 1] = im + (b * re + a * im);
                    } else {
                        tmp[2 * y] = a * re - b * im;
                        tmp[2 * y + 1] = b * re + a * im;
                    }
                }
                for (int y = 0; y < d->S; y++) {
                    int i = 2 * d->D + y;
                    tmp[i] = d->residual ? v[i] + d->sfwd[y] * v[i] : d->sfwd[y] * v[i];
                }
                memcpy(v, tmp, N * sizeof(double));
            }
        }
        memcpy(out + (size_t)t * N, v, N * sizeof(double));
    }
    free(Om);
    free(v);
    free(pt.row_ptr);
    free(pt.col);
    return 0;
}

/* Simulate ntraj independent trajectories (sharing generators, differing
 * in their coefficient programs and initial states).
 *   progs: ntraj * nch * nseg * 5   rho0: ntraj * N   out: ntraj * T * N
 * For rotating runs rho0/out are in the rotating eigenbasis in vector mode
 * (the caller transforms), and in the lab basis in reference mode (the
 * sandwich is applied to the propagators, as the reference does).
 * Returns 0, or -1 on allocation failure, -2 on bad arguments. */
int sss_oracle_simulate(int N, int G, int K, int Q, const double* gens,
                        const double* W, const double* nodes, int rotating,
                        const double* dfwd, int D, const double* sfwd, int S,
                        const double* V, const double* Vinv, int residual,
                        int R, int degree, const double* progs, int nch,
                        int nseg, double t0, double dt, int T, int F,
                        int ntraj, const double* rho0, double* out, int mode,
                        int threads) {
    if (N <= 0 || G <= 0 || G > 16 || K <= 0 || Q <= 0 || Q * G > 64 || T < 0 ||
        F <= 0 || ntraj < 0)
        return -2;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    int status = 0;
    if (mode == SSS_ORACLE_REFERENCE) {
        for (int b = 0; b < ntraj && status == 0; b++) {
            oracle_desc d = {N, G, K, Q, gens, W, nodes, rotating, dfwd, D, sfwd, S, V,
                             Vinv, residual, R, degree,
                             progs + (size_t)b * nch * nseg * 5, nch, nseg};
            status = run_reference(&d, t0, dt, T, F, rho0 + (size_t)b * N,
                                   out + (size_t)b * T * N);
        }
    } else {
#pragma omp parallel for schedule(dynamic, 1) reduction(min : status)
        for (int b = 0; b < ntraj; b++) {
            oracle_desc d = {N, G, K, Q, gens, W, nodes, rotating, dfwd, D, sfwd, S, V,
                             Vinv, residual, R, degree,
                             progs + (size_t)b * nch * nseg * 5, nch, nseg};
            int s = run_vector(&d, t0, dt, T, F, rho0 + (size_t)b * N,
                               out + (size_t)b * T * N);
            if (s < status) status = s;
        }
    }
    return status;
}

int sss_oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
