/*
 * sss.h -- C-ABI of libsss.so, the GB300 (sm_103a) time-stepping core of
 * superspinsim_gb300.
 *
 * The reference (monashNV/superspinsim 1.3.2) is pure Python: its hot path
 * is the closure built by `generate_simulator(...)`
 * (superspinsim/generate_simulator.py:17-154) and the `simulate(rho0, t0,
 * tf, dt)` function it returns (:1508-2200), whose device work is a set of
 * numba.cuda kernels launched from Python.  A Python caller of this library
 * (superspinsim_gb300/generate_simulator.py, through ctypes) keeps that
 * API; these entry points replace the numba kernels and their host driver
 * loop:
 *
 *   sss_plan_create    replaces generate_simulator's set-up
 *                      (:49-154: flag handling, 4^R scaling, CF table
 *                      selection, generator cast and upload :1697-1811)
 *   sss_plan_set_rotating  the generalised-rotating-frame set-up
 *                      (:142-151, host frame preparation :1567-1677)
 *   sss_simulate       `simulate` (:1508-2200) for one or more trajectories:
 *                      the fine-step loop :1954-2015, the chain :2025-2028,
 *                      the frame sandwich :2030-2038 and rho(t) = U(t) rho0
 *                      :2111-2116.  Host buffers in and out.
 *   sss_simulate_device  the same on device pointers (inputs resident in
 *                      HBM), for callers that own device memory.
 *   sss_batch_run      no single reference counterpart: the batched sweep
 *                      that replaces calling `simspins` in a loop
 *                      (superspinsim/sugar.py:566-583) once per parameter
 *                      point.  Persistent kernel, device work queue.
 *   sss_last_error / sss_plan_destroy   error text and teardown.
 *
 * Conventions.  All arithmetic is IEEE binary64.  Matrices are row-major.
 * A state is the real vectorised density operator of length N in the
 * reference's Hermitian basis (vectorisation_map rows (y, x, c),
 * superspinsim/generate_generators.py:2361-2382).  Every entry point
 * returns 0 on success or a negative SSS_E* code; nothing aborts or throws
 * across the ABI, and sss_last_error() gives a thread-local message.
 * A plan owns its device memory; host buffers stay caller-owned and are
 * only touched during the call.  A plan is not thread-safe: use one plan
 * per host thread.
 */
#ifndef SSS_H
#define SSS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SSS_OK 0
#define SSS_EINVAL (-1)     /* bad shape or argument */
#define SSS_ENOMEM (-2)     /* device or host allocation failed */
#define SSS_ECUDA (-3)      /* a CUDA call failed */
#define SSS_ETIMEOUT (-4)   /* a device wait ran out of iterations (reserved:
                               no kernel of this library waits on a flag --
                               the work queue is a bare atomic counter) */
#define SSS_ENONFINITE (-5) /* a state became NaN or infinite */
#define SSS_ENODEVICE (-6)  /* no CUDA device */

/* plan flags */
#define SSS_RESIDUAL 1u     /* residual arithmetic (accumulate U - I) */
#define SSS_ROTATING 2u     /* generalised rotating frame */

/* exponential algorithms */
#define SSS_EXPM_REFERENCE 0 /* first-order Taylor, 4^-R scaling, 2R squarings
                                (generate_simulator.py:534-578, :706-724) */
#define SSS_EXPM_TAYLOR 1    /* Taylor of chosen degree, norm-chosen squarings */

typedef struct sss_plan sss_plan;

typedef struct {
    int N;          /* vectorised dimension */
    int G;          /* generators: lab frame [L0, Gx, Gy, Gz, Gr] (5),
                       rotating frame [Gx, Gy, Gz, Gr] (4) */
    int K;          /* exponentials per step (1, 2, 3, 5, 6) */
    int Q;          /* Gauss-Legendre nodes (1, 2, 3) */
    unsigned flags; /* SSS_RESIDUAL | SSS_ROTATING */
    int expm;       /* SSS_EXPM_REFERENCE or SSS_EXPM_TAYLOR */
    int quartic_repeats; /* R: 2R squarings in SSS_EXPM_REFERENCE */
    int taylor_degree;   /* SSS_EXPM_TAYLOR degree (0: chosen per run) */
} sss_plan_desc;

/* generate_simulator set-up.  generators: G*N*N (lab frame; unused and
 * may be NULL with SSS_ROTATING, whose per-node generators come from
 * sss_plan_set_rotating).  weights: K*Q commutator-free weights; nodes: Q
 * Gauss-Legendre nodes in [0, 1]. */
int sss_plan_create(sss_plan** plan, const sss_plan_desc* desc,
                    const double* generators, const double* weights,
                    const double* nodes);

/* Rotating frame (generate_simulator.py:1567-1677, 901-1021, 1023-1171):
 * generators_nodes: Q*G*N*N rotating generators at each node offset;
 * doubles_last: D*2 and singles_last: S, the residual-aware (or plain)
 * e^{L0 h} blocks for one fine step; V, Vinv: N*N eigenbasis and its
 * inverse.  2D + S == N.  The fine step h is fixed by these tables: a run
 * must use the dt/F they were made for. */
int sss_plan_set_rotating(sss_plan* plan, const double* generators_nodes,
                          const double* doubles_last, int D,
                          const double* singles_last, int S, const double* V,
                          const double* Vinv);

/* Coefficient program of one trajectory: nch channels x nseg segments x 5
 * doubles (t_end, offset, amplitude, frequency, phase).  A channel's value
 * at time t is offset + amplitude*cos(tau*frequency*t + phase) for the
 * first segment with t < t_end, else 0.  Lab frame: coefficient row
 * [1, ch0, ch1, ch2, ch3]; rotating frame: [ch0, ch1, ch2, ch3]
 * (superspinsim/generate_generators.py:2317-2358). */

/* simulate() for ntraj independent trajectories, host buffers.
 *   rho0:  ntraj*N          flattened initial states
 *   programs: ntraj*nch*nseg*5, or NULL when coeff_table is given
 *   coeff_table: ntraj*(T*F*Q)*G sampled coefficients in the reference's
 *          row order (sample t, node k at fine step r in row
 *          (r*T + t)*Q + k), or NULL
 *   out:   ntraj*T*N  state after each of the T output samples
 * Output sample t is at t0 + dt*(t+1); each spans F fine steps of dt/F. */
int sss_simulate(sss_plan* plan, int ntraj, const double* rho0, int nch,
                 int nseg, const double* programs, const double* coeff_table,
                 double t0, double dt, int T, int F, double* out,
                 void* cuda_stream);

/* The same with every pointer a device pointer. */
int sss_simulate_device(sss_plan* plan, int ntraj, const double* rho0, int nch,
                        int nseg, const double* programs,
                        const double* coeff_table, double t0, double dt, int T,
                        int F, double* out, void* cuda_stream);

/* Batched sweep: ntraj trajectories, each with its own program, initial
 * state and number of output samples, run by a persistent kernel that
 * takes trajectories from a device work queue.  Per output sample t of
 * trajectory b it writes readout[b*T_max + t] = dot(readout_weights, state)
 * (a linear functional such as a population or a fluorescence rate); after
 * its last sample the row is zero-padded.  final_state (ntraj*N) receives
 * each trajectory's last state (NULL to skip); trace (ntraj*T_max*N)
 * receives the full state after every output sample (NULL to skip; zero
 * after a trajectory's last sample).
 *   samples: ntraj output-sample counts (NULL: all T_max)
 *   host != 0: all pointers are host pointers (copied in and out within the
 *   call); host == 0: device pointers.
 * Uses SSS_EXPM_TAYLOR arithmetic.  A rotating plan (SSS_ROTATING, tables
 * set) runs in the generalised rotating frame on the row-part kernel
 * (variant 0 or 4): states, weights and outputs stay in the lab basis, the
 * kernel converting with V and V^-1 (generate_simulator.py:450-532 Omega,
 * :901-1021 e^{L0 h} blocks, :2030-2038 sandwich).
 * Health check (the reference has none): the kernels test every readout
 * and final-state value they write and record the first NaN or infinity
 * in a device word.  With host != 0 the call returns SSS_ENONFINITE
 * (naming the trajectory and output sample) when one was written; with
 * host == 0 the call stays asynchronous and sss_batch_check reports it. */
int sss_batch_run(sss_plan* plan, int ntraj, const double* rho0, int nch,
                  int nseg, const double* programs, const int* samples,
                  double t0, double dt, int T_max, int F,
                  const double* readout_weights, double* readout,
                  double* final_state, double* trace, int host,
                  void* cuda_stream);

/* sss_batch_run with sampled coefficients instead of programs: the
 * fallback for arbitrary samplers (the reference's sampler callables,
 * generate_simulator.py:235-271, evaluated by the caller).
 *   coeff_table: ntraj*(F*T_max*Q)*G, per trajectory the rows of
 *          sss_simulate's table with T = T_max: row (r*T_max + t)*Q + k
 *          holds the G coefficients (lab [c_L0, c_1, ...], rotating
 *          [c_1, ...]) at node k of fine step r of output sample t.
 * Runs on the row-part kernel (variant 0 or 4).  A column that holds one
 * value everywhere is folded into the constant part of Omega; the Taylor
 * degree follows the table's largest |coefficient| per column.  NaN or
 * infinity anywhere in the table is SSS_ENONFINITE.  The other arguments
 * are sss_batch_run's. */
int sss_batch_run_table(sss_plan* plan, int ntraj, const double* rho0,
                        const double* coeff_table, const int* samples,
                        double t0, double dt, int T_max, int F,
                        const double* readout_weights, double* readout,
                        double* final_state, double* trace, int host,
                        void* cuda_stream);

/* The batched run in two parts (no reference counterpart).
 * sss_batch_prepare analyses the batch on the host -- active generators,
 * rows reachable from rho0's support, lane layout, Taylor degree from the
 * programs' amplitude bound -- and uploads the kernel's tables (device
 * pointers; readout_weights is a host array of N or NULL).  The prepared
 * state lives in the plan until the next prepare or batched run.
 * sss_batch_launch then runs output samples [t_begin, t_begin + n_samples)
 * of every trajectory, continuing in place from `state` (ntraj*N, device:
 * in, the states at sample t_begin; out, the states after the chunk) and
 * filling those columns of `readout` (ntraj*T_max, or NULL).  It does not
 * allocate or synchronise with the host, so a sequence of launches can be
 * captured in a CUDA graph; chunks make runs resumable.  Programs passed to
 * a launch may change values but must keep the prepared batch's size,
 * shape, dt and F, the same zero/non-zero channels, no larger amplitudes
 * (the Taylor degree was chosen for them) and initial states within the
 * prepared support. */
int sss_batch_prepare(sss_plan* plan, int ntraj, const double* rho0, int nch,
                      int nseg, const double* programs, double dt, int F,
                      const double* readout_weights, void* cuda_stream);
/* sss_batch_prepare for trajectories of uneven length: `samples` (host,
 * ntraj) holds each trajectory's output-sample count, and every
 * sss_batch_launch of the prepared batch must pass the same counts (as a
 * device array).  Trajectories are then handed out longest first and,
 * with automatic lanes (variant 0 or 4), the batch is also laid out for
 * the wider lane groups that the trajectories still running call for as
 * the shorter ones finish: a launch switches layout at the output samples
 * where the running count stops filling the GPU, and cuts its grid to the
 * trajectories still running, without allocating or synchronising (the
 * chunks stay graph-capturable).  sss_batch_run does this by itself when
 * it is given samples. */
int sss_batch_prepare_samples(sss_plan* plan, int ntraj, const double* rho0,
                              int nch, int nseg, const double* programs,
                              const int* samples, double dt, int F,
                              const double* readout_weights, void* cuda_stream);
int sss_batch_launch(sss_plan* plan, double* state, const double* programs,
                     const int* samples, double t0, int t_begin, int n_samples,
                     int T_max, double* readout, void* cuda_stream);
/* Synchronises cuda_stream and reads the health word of the prepared batch:
 * SSS_ENONFINITE if a launch (or device-pointer sss_batch_run) since the
 * last prepare or check wrote a NaN or infinite readout or final-state
 * value (the word is then reset), else SSS_OK.  Call it after the last
 * chunk of a run, or after replaying a captured graph of launches. */
int sss_batch_check(sss_plan* plan, void* cuda_stream);

/* Adjoint gradients (no reference counterpart: the reference computes no
 * derivatives).  For each trajectory, the objective
 *   J = sum_t time_weights[t] * dot(readout_weights, state after sample t)
 * (for example integrated fluorescence: excited populations times the
 * decay rate, trapezoid weights over the readout window) and its gradient
 * with respect to the amplitude and phase of every segment of channel 0
 * (the x field):  grad[(b*nseg + s)*2 + 0] = dJ/d amplitude_s,
 * grad[(b*nseg + s)*2 + 1] = dJ/d phase_s.  The forward pass stores the
 * state before every exponential (trajectories in chunks that fit the
 * memory bound of sss_plan_set_adjoint_memory) and the backward sweep walks
 * them back; when the states of one trajectory do not fit, a checkpointed
 * sweep (about sqrt(T*F) checkpoints, each interval recomputed) runs
 * instead.  The exponential's derivative is exact for the truncated series
 * the forward pass uses.  Lab frame.  readout_weights (N) and time_weights
 * (T) are host arrays; the rest follow `host` as in sss_batch_run. */
int sss_adjoint_run(sss_plan* plan, int ntraj, const double* rho0, int nch,
                    int nseg, const double* programs, double t0, double dt,
                    int T, int F, const double* readout_weights,
                    const double* time_weights, double* J, double* grad,
                    int host, void* cuda_stream);

/* sss_adjoint_run for the segments of any program channel, with four
 * parameters per segment: channel c (0 <= c < nch, generator G_{c+1}; 3 is
 * the fourth channel, e.g. the laser power) and
 *   grad[((b*nseg + s)*4 + 0]  dJ/d amplitude_s
 *   grad[((b*nseg + s)*4 + 1]  dJ/d phase_s
 *   grad[((b*nseg + s)*4 + 2]  dJ/d offset_s
 *   grad[((b*nseg + s)*4 + 3]  dJ/d frequency_s
 * of c(t) = offset_s + amplitude_s cos(2 pi frequency_s t + phase_s).  The
 * other channels are held fixed.  SSS_EINVAL when the channel has no
 * generator or its generator is zero on the rows reachable from rho0;
 * with host != 0, SSS_ENONFINITE when J or a gradient entry is NaN or
 * infinite.  sss_adjoint_run is channel 0 with the first two entries. */
int sss_adjoint_run_channel(sss_plan* plan, int ntraj, const double* rho0,
                            int nch, int nseg, const double* programs,
                            double t0, double dt, int T, int F,
                            const double* readout_weights,
                            const double* time_weights, int channel,
                            double* J, double* grad, int host,
                            void* cuda_stream);

/* Equivalence-class ("kernel") mode.  The plan's generators act on the
 * r = N dimensional image of the orthonormal basis P (n_full x N, row-major),
 * the complement of the generators' common kernel.  sss_simulate and
 * sss_simulate_device then take and return states of n_full entries:
 * rho(t) = rho0 + P (U_r(t) - I) P^T rho0, i.e. the full propagator
 * P U_r P^T + (I - P P^T), with the common-kernel components held fixed.
 * Replaces the reference's equivalence-class sandwich and kernel addition
 * (generate_simulator.py:1789-1797, 2043-2071), whose residual sandwich reads
 * out of bounds (:1047); this is the form it intends.  n_full = 0 clears the
 * mode.  Batched runs and the adjoint reject projected plans. */
int sss_plan_set_projection(sss_plan* plan, int n_full, const double* image_projection);

/* Unitary mode.  The plan's N = 2n generators are real forms of n x n
 * complex matrices (entry (i, j) at [2i][2j] real and [2i+1][2j] imaginary,
 * generate_generators.py:2725-2746), so the integrator propagates an
 * operator U.  sss_simulate then returns densities conj(U) rho0 U^T -- what
 * the reference's Kronecker product, unitary copy and elimination /
 * duplication sandwich produce (generate_simulator.py:1394-1504, 2074-2101),
 * without its out-of-bounds reads (:1026) -- flattened by `map` (nd rows
 * y, x, c as the vectorisation map; rho0 is read the same way, off-diagonal
 * rows mirrored to their Hermitian partner) or, with map = NULL, all 2n^2
 * entries row-major.  With the reference's generators (the real form of
 * +iH) this is the unitary evolution of the Liouvillian mode whenever H is
 * real.  n = 0 clears the mode.  Batched runs and the adjoint reject
 * unitary plans. */
int sss_plan_set_unitary(sss_plan* plan, int n, int nd, const int* map);

/* Kernel launches issued by the last sss_simulate / sss_batch_run call on
 * this plan (for launch accounting). */
int sss_plan_last_launches(const sss_plan* plan);

/* Batched-kernel configuration (the autotuner's knobs): lanes per
 * trajectory (1, 2, 4, ..., 256; 0 = automatic; above 32 the row-part
 * variant only, one trajectory per CTA of that many threads), CTA size (a multiple of
 * 32 up to 256; 0 = 32 for the row-part variant, else 64) and variant
 * (0 = automatic: the row-part variant when the pattern fits, else as 1;
 * 1 = register variant when the per-lane share fits, else shared memory;
 * 2 = always the shared-memory variant; 3 = register variant with one FMA
 * chain per row; 4 = row-part variant: rows cut into parts of a few
 * entries, each lane running C equal-length FMA chains, 8, 16 or 32 lanes,
 * small patterns only -- SSS_EINVAL when the pattern does not fit; 5 = as
 * 4, with the state in registers moved by warp shuffles where the layout
 * allows it: 32 lanes, one chain per lane, no lane owning two rows, lab
 * frame; 6 = slot-packed: every lane runs the same S FMA slots per Horner
 * term in scaled Horner form (the v term of a row is one more entry), rows
 * of n entries taking n + 1 slots with no padding to a part length
 * (sss_slot_layout), 8 to 256 lanes, up to 16 slots; 7 = phased row parts:
 * per lane C1 chains of P1 slots, a barrier, then C2 chains of P2 slots
 * that start from parked partial sums, every chain starting at a fixed
 * slot, 8, 16 or 32 lanes).  Automatic lanes: per lane count the cheapest
 * layout (FP64 instructions per Horner term), and the lane count whose
 * busiest SM sub-partition issues the fewest of them.  Configured lanes
 * also set the adjoint's forward and backward groups; for sss_adjoint_run
 * variant 4 or 5 selects the row-part backward, the others the
 * slot-programmed backward (the block series [[Omega^T, G^T], [0, Omega^T]]
 * on a slot program) where it fits, and variant 1 the checkpointed
 * adjoint.  No
 * reference counterpart (the reference's launch shapes are fixed,
 * generate_simulator.py:85-106). */
int sss_plan_set_batch_config(sss_plan* plan, int lanes, int cta_threads,
                              int variant);

/* Device memory (bytes) sss_adjoint_run may use for the forward states it
 * stores (the state before every exponential of every trajectory); 0 = half
 * of the free device memory at the call.  Trajectories are processed in
 * chunks that fit; when the states of one trajectory do not fit, the
 * checkpointed adjoint (which recomputes intervals) runs instead.  No
 * reference counterpart (the reference has no derivatives). */
int sss_plan_set_adjoint_memory(sss_plan* plan, size_t max_bytes);

/* What the last sss_batch_run used: lanes per trajectory, Taylor degree,
 * sub-steps per exponential, state rows kept after the reachability
 * pruning, non-zeros of the pruned pattern, and the kernel's device time in
 * ms (CUDA events on the launch stream; waits for it).  Any pointer may be
 * NULL. */
int sss_plan_batch_info(const sss_plan* plan, int* lanes, int* degree,
                        int* substeps, int* rows, int* nnz, double* kernel_ms);

/* Layout utility (no reference counterpart; host only, needs no device):
 * the slot-packed layout that batched runs use (variant 6) for a row
 * pattern of M rows, row i holding columns col[row_ptr[i] .. row_ptr[i+1])
 * (state rows of Omega's non-zeros), at `lanes` lanes per trajectory (8 to
 * 256) and at most max_slots slots per lane (capped at 16).  Every lane runs
 * the same `slots` FMA instructions per Horner term: a row of n entries
 * takes n entry slots and one close slot (its v term), and a row cut
 * between two lanes parks a partial sum before slot `barrier_slot` (equal
 * to `slots` when no row is cut) that the other lane picks up there or
 * later.  words and entries (16*lanes values each, [slot*lanes + lane])
 * receive each slot's word -- bits 0-13 the state row it reads (an entry; a
 * partial index for a partial add) or closes (a close), bit 14 partial add,
 * bit 15 close, bit 16 piece start, bit 17 start from partial `pidx`, bit
 * 18 park the sum as partial `pidx`, bits 19-31 pidx -- and the index into
 * col of the entry it multiplies (-1: close or padding, -2: partial add).
 * SSS_EINVAL when no layout of at most max_slots slots exists. */
int sss_slot_layout(int M, const int* row_ptr, const int* col, int lanes,
                    int max_slots, int* slots, int* barrier_slot, int* partials,
                    unsigned* words, int* entries);

/* What the last batched run executes (no reference counterpart; for the
 * roofline count): the kernel variant chosen (1-7, as
 * sss_plan_set_batch_config), the generators assembled per exponential
 * (those whose coefficient varies; the constant ones are folded into a
 * table), their non-zeros on the pruned pattern, and the FP64 instructions
 * one group issues per Horner term.  Any pointer may be NULL. */
/* Shared-memory bank conflicts of the last slot-programmed layout (variants
 * 6 and 7; no reference counterpart): the extra wavefronts one Horner term
 * of one group costs, as modelled on the host from the layout's loads and
 * stores (per half-warp and instruction, the distinct 8-byte words beyond
 * one per bank), with the rows numbered in lane order (before) and after
 * the bank-aware renumbering the layout runs with (after).  Any pointer
 * may be NULL. */
int sss_plan_bank_conflicts(const sss_plan* plan, int* before, int* after);

int sss_plan_batch_work(const sss_plan* plan, int* variant, int* live_generators,
                        int* live_nnz, int* fp64_per_term);

/* Measurement utility (no reference counterpart): FP64 FMA throughput of
 * the current device in TFLOP/s, from a bounded DFMA loop (8 independent
 * chains per thread, 4 CTAs of 256 threads per SM).  The roofline
 * denominator of the FP64-bound kernels. */
int sss_fp64_peak(double* tflops, void* cuda_stream);

/* Measurement utility (no reference counterpart): FP64 tensor-core (DMMA,
 * mma.sync m8n8k4 f64) throughput in TFLOP/s from a bounded loop over 8
 * independent accumulator tiles per warp, 4 CTAs of 256 threads per SM.
 * Reported beside sss_fp64_peak: on GB300 it is below the DFMA rate, which
 * is why no kernel here uses the FP64 tensor path. */
int sss_fp64_mma_peak(double* tflops, void* cuda_stream);

/* Allocation-free simulate for one trajectory (no counterpart in the
 * reference, which always allocates per call).  For callers that cannot
 * allocate device memory -- code inside another framework's memory pool, a
 * device whose memory is already reserved, or a context where allocation is
 * not allowed.  It runs the plain path's kernels with a fixed 4 MiB
 * file-scope device array as scratch and allocates nothing.
 *   desc: N <= 52, lab frame (SSS_ROTATING rejected); generators (G*N*N),
 *   rho0 (N), programs (nch*nseg*5) and out (T*N) are device pointers;
 *   weights (K*Q) and nodes (Q) are host pointers.
 * Every GPU that loads the library holds the array until exit.  All calls
 * share it, so calls that overlap on the GPU race.  The first call on a
 * device looks up the array's address there; make it before any stream
 * capture.  Sizes beyond the limit return SSS_EINVAL with a message. */
int sss_simulate_noalloc(const sss_plan_desc* desc, const double* generators,
                         const double* weights, const double* nodes,
                         const double* rho0, int nch, int nseg,
                         const double* programs, double t0, double dt, int T,
                         int F, double* out, void* cuda_stream);

const char* sss_last_error(void);
void sss_plan_destroy(sss_plan* plan);

#ifdef __cplusplus
}
#endif
#endif /* SSS_H */
