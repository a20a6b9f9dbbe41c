// Internal declarations shared by the translation units of libsss.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <unordered_map>
#include <vector>

#include "sss.h"
#include "sss_lanes.h"

namespace sss {

constexpr double kTau = 6.283185307179586;
constexpr int kMaxG = 8;      // generators per frame
constexpr int kMaxQ = 3;      // Gauss-Legendre nodes
constexpr int kMaxK = 6;      // exponentials per step
constexpr int kMaxCh = 4;     // coefficient channels
constexpr int kMaxSlots = kMaxQ * kMaxG;
constexpr int kMaxPhases = 6;  // lane counts of a prepared batch (8 .. 256)  // generator slots of a rotating plan (node, generator)
constexpr int kPlainMaxN = 52;  // dense shared-memory propagator path
// row-part kernels (forward and adjoint)
constexpr int kCloseMax = 8;    // close slots per lane
constexpr int kRing = 16;       // fine steps of coefficients per refill
// (C parts per lane, P entries per part) shapes instantiated
constexpr int kPartShapes[][2] = {{1, 4}, {2, 4}, {4, 4}, {2, 8}};
// slot-packed kernels: slots per lane (S <= kSlotsMax)
constexpr int kSlotsMax = 16;

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define SSS_CUDA(call)                                      \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return sss::cuda_fail(e_, #call); \
    } while (0)

// Device buffer that grows on demand and is owned by a plan.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t n);
    void release();
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// Sparse form of the generators for the batched vector-action kernel:
// the union pattern of all generators, row-sorted.  For each pattern entry
// p: row, col, and the G generator values at (row, col).
struct SparseGenerators {
    int N = 0, G = 0, nnz = 0;
    std::vector<int> row_ptr;   // N+1
    std::vector<int> col;       // nnz
    std::vector<double> val;    // G*nnz, generator-major
};

// Host-side layout of the batched kernels: reachable rows, active
// generators, rows split across L lanes, per-lane entry lists.
struct BatchLayout {
    struct Ent { int col; int q; };   // compressed column, index into SparseGenerators
    int M = 0, Ga = 0, L = 0, E = 0, epl = 0, degree = 0, substeps = 0, threads = 0;
    bool use_reg = false;
    long nnz = 0;
    std::vector<int> active;                 // active generator indices
    std::vector<std::vector<Ent>> row_ents;  // per reachable row (reachable order)
    std::vector<std::vector<int>> lane_of;   // rows (reachable order) of each lane
    std::vector<int> newpos, row_orig;       // reachable -> lane order; lane order -> original
    std::vector<double> gv;                  // Ga*E*L generator values [g][e][l]
    std::vector<unsigned> words;             // E*L entry words [e][l]
    std::vector<int> entry_q;                // E*L index into SparseGenerators (-1: padding,
                                             // -2: partial add, -3: constant entry, value in cval)
    std::vector<double> cval;                // E*L constant entries' values (slot layouts)
    std::vector<int> cnt;                    // entries of each lane
    // row-part variant: C parts of P entries per lane, kc close slots
    bool parts = false;
    int C = 0, P = 0, kc = 0;
    std::vector<int> pcol;                   // C*P*L part entry columns [e][l]
    std::vector<unsigned> cw;                // kCloseMax*L close words [k][l]
    // slot-packed and phased row-part variants: S FMA slots per lane per
    // Horner term, kernel slot words in cw (load words [q][l], then store
    // words [S+q][l]), a barrier before slot bar_at, npart parked partial
    // sums per trajectory; phased: the shape index into kPhasedShapes
    bool slots = false, phased = false;
    int S = 0, bar_at = 0, npart = 0, shape = 0;
    std::vector<char> chan_const;            // per generator slot: its channel is batch-constant
    std::vector<double> chan_value;          // that constant
    std::vector<int> slot_chan;              // per generator slot: its program channel (-1: L0)
};

}  // namespace sss

struct sss_plan {
    sss_plan_desc d{};
    double W[sss::kMaxK * sss::kMaxQ] = {};
    double nodes[sss::kMaxQ] = {};
    bool rotating = false;
    int D = 0, S = 0;
    // host copies
    std::vector<double> gens;        // lab G*N*N, or rotating Q*G*N*N
    std::vector<double> dlast, slast, V, Vinv;
    sss::SparseGenerators sparse;    // lab frame, for sss_batch_run
    // device copies
    sss::DevBuf d_gens, d_dlast, d_slast, d_V, d_Vinv;
    sss::DevBuf d_sp_rowptr, d_sp_col;
    sss::DevBuf d_row_map;
    // workspace
    sss::DevBuf w_prop, w_in, w_out, w_prog, w_tab, w_aux, w_queue, w_ro,
        w_fin, w_samples, w_status;
    // health word of the prepared batch (see BatchArgs::health), reset by
    // sss_batch_prepare and by a check that found an error
    sss::DevBuf w_health;
    int last_launches = 0;
    int batch_lanes = 0;    // 0: chosen per run
    int batch_threads = 0;  // CTA size of the batched kernel, 0: 128
    int last_batch_lanes = 0, last_degree = 0, last_substeps = 0, last_rows = 0,
        last_nnz = 0, last_grid = 0, last_epl = 0, last_active = 0, last_variant = 0;
    // executed work of the last prepared batch (phase 0): generators assembled
    // per exponential, their non-zeros on the pruned pattern, FP64
    // instructions per Horner term per group; make_args records the first two
    int last_n_live = 0, last_live_nnz = 0, last_fp64_per_term = 0, mk_n_live = 0, mk_live_nnz = 0;
    // bank-aware renumbering of slot-programmed layouts: the modelled extra
    // shared-memory wavefronts of one Horner term (one group) before and
    // after, for the last layout built, and the numberings found so far
    // (keyed by a hash of the layout's kernel words)
    int last_bank_before = 0, last_bank_after = 0;
    // values of the constant entries of a slot layout being built: an entry
    // whose q is sparse.nnz + k has the fixed value slot_consts[k] and no
    // generator values (the G^T block of the adjoint's block series)
    std::vector<double> slot_consts;
    std::unordered_map<uint64_t, std::vector<int>> bank_cache;
    int batch_variant = 0;  // 0: register variant when it fits, 2: shared-memory variant,
                            // 3: one-chain register variant, 4: row-part variant
    int device = 0;
    int num_sms = 0;
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;  // around the last batched run's kernels
    bool ev_recorded = false;
    bool ev_keep_begin = false;  // a later phase of one run: keep the first launch's begin event
    int auto_lanes_ntraj = 0;    // trajectories the automatic lane rule counts (0: the batch)
    double auto_cost[sss::kLaneCounts] = {};  // last automatic layout: cost per lane count 8..256
    int launch_active = 0;       // trajectories with work in the next launch (0: the batch)
    // prepared batch (sss_batch_prepare -> sss_batch_launch): one kernel
    // layout per phase -- a single phase, or with uneven lengths and
    // automatic lanes one per widening lane count, phase k running from
    // output sample t_start on
    struct BatchPhase {
        alignas(16) unsigned char args[1536];
        size_t smem = 0;
        int L = 0, C = 0, P = 0, epl = 0, threads = 0, t_start = 0, S = 0, shape = 0;
        bool use_reg = false, one_chain = false, parts = false, shfl = false, slots = false,
             phased = false;
    };
    BatchPhase batch_phase[sss::kMaxPhases];
    sss::DevBuf batch_tables[sss::kMaxPhases];
    int batch_nphases = 0;
    std::vector<int> batch_longest;    // the prepared sample counts, longest first (or empty)
    const int* batch_order = nullptr;  // queue position -> trajectory, longest first (w_order)
    bool batch_ready = false, batch_empty = false, batch_has_rw = false, batch_table = false;
    int batch_ntraj = 0, batch_nch = 0, batch_nseg = 0, batch_F = 0;
    double batch_dt = 0.0;
    sss::DevBuf w_state;
    // adjoint (row-part path): forward and backward tables, stored states,
    // readouts, state buffer
    sss::DevBuf w_adjf, w_adjb, w_states, w_adjro, w_adjst, w_order;
    size_t adj_max_bytes = 0;  // stored-state memory of the adjoint, 0: half the free memory
    // equivalence-class (kernel) mode: states of n_full entries, image basis P
    // (n_full x N); unitary mode: operator generators of a u_n-level system
    // (N = 2 u_n), densities of u_nd entries (map u_map rows y, x, c, or all
    // 2 u_n^2 entries row-major)
    int n_full = 0;
    sss::DevBuf d_P;
    int u_n = 0, u_nd = 0;
    bool u_mapped = false;
    sss::DevBuf d_umap;
    // entries of one input state and of one output sample of sss_simulate
    int state_in() const { return n_full ? n_full : (u_n ? u_nd : d.N); }
};

namespace sss {
// sss_plain.cu
int plain_run(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg,
              const double* d_prog, const double* d_tab, double t0, double dt,
              int T, int F, double* d_out, cudaStream_t st);
// sss_batch.cu
int batch_run(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg,
              const double* d_prog, const int* d_samples, const int* h_samples,
              double t0, double dt, int T_max, int F, const double* h_rw,
              double* d_readout, double* d_final, cudaStream_t st, double* d_trace = nullptr,
              const double* d_tab = nullptr);
int build_sparse(sss_plan* p);
// sss_adjoint.cu
// dch: the differentiated channel; npar: 2 (amplitude, phase) or 4 (also
// offset, frequency) gradient entries per segment
int adjoint_run(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg,
                const double* d_prog, double t0, double dt, int T, int F, const double* h_rw,
                const double* h_tw, int dch, int npar, double* d_J, double* d_grad,
                cudaStream_t st);
// d_tab: a coefficient table (ntraj*(F*T_tab*Q)*G, rows (r*T_tab + t)*Q + k)
// in place of the programs; it runs on the row-part kernel
// h_samples: the trajectories' output-sample counts (host), or null; with
// them trajectories are handed out longest first and, with automatic lanes,
// the batch is prepared in phases
int batch_prepare(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg,
                  const double* d_prog, double dt, int F, const double* h_rw, cudaStream_t st,
                  const double* d_tab = nullptr, int T_tab = 0, const int* h_samples = nullptr);
int batch_launch(sss_plan* p, double* d_state, const double* d_prog, const int* d_samples,
                 double t0, int t_begin, int n_samples, int T_max, double* d_readout,
                 cudaStream_t st, double* d_trace = nullptr, const double* d_tab = nullptr);
// Waits for the stream and reads the prepared batch's health word:
// SSS_ENONFINITE (and the word reset) if a launch since the last prepare or
// check wrote a NaN or infinite readout or final-state entry.
int batch_check(sss_plan* p, cudaStream_t st);
int build_layout(sss_plan* p, int ntraj, const double* d_rho0, int nch, int nseg,
                 const double* d_prog, double dt, int F, const std::vector<int>& force_active,
                 bool allow_register, BatchLayout* out, cudaStream_t st, bool force_parts = false,
                 const double* d_tab = nullptr, int T_tab = 0);
int slot_layout_host(int M, const int* row_ptr, const int* col, int L, int S_cap, int* S_out,
                     int* bar_out, int* npart_out, unsigned* words, int* entries);
// Slot-packed and phased row-part layouts of given rows (entries with q >=
// sparse.nnz are constant entries, see sss_plan::slot_consts), and the
// bank-aware placement of such a layout (varies[g]: generator slot g is
// assembled every exponential).
int slots_layout_rows(sss_plan* p, const std::vector<std::vector<BatchLayout::Ent>>& rows, int L,
                      int threads, int S_cap, const std::vector<int>& active,
                      const std::vector<int>& rows_reached, BatchLayout* out);
int phased_layout_rows(sss_plan* p, const std::vector<std::vector<BatchLayout::Ent>>& rows, int L,
                       int threads, int S_cap, const std::vector<int>& active,
                       const std::vector<int>& rows_reached, const std::vector<char>& varies,
                       BatchLayout* out);
int place_banks(sss_plan* p, BatchLayout& Ly, const std::vector<int>& active,
                const std::vector<char>& varies);
int parts_layout_rows(sss_plan* p, const std::vector<std::vector<BatchLayout::Ent>>& rows,
                      const std::vector<std::vector<char>>& prio, int L, int threads, int w_chain,
                      int w_close, const std::vector<int>& active,
                      const std::vector<int>& rows_reached, BatchLayout* out, int* nprio);
// Row-part forward kernel prepared outside the plan's batch state (for the
// adjoint): opaque kernel arguments and launch shape.
struct PartsForward {
    alignas(16) unsigned char args[1536];
    size_t smem = 0;
    int L = 0, C = 0, P = 0, threads = 0;
};
// Build the device tables of a row-part layout into `tables` and the
// forward kernel's arguments.  Generators in `keep_live` are never folded
// into the constant part of Omega.
int parts_forward_prepare(sss_plan* p, const BatchLayout& Ly, int ntraj, int nch, int nseg,
                          double dt, int F, const double* h_rw, const std::vector<int>& keep_live,
                          DevBuf& tables, PartsForward* fw, cudaStream_t st);
// Launch it on `ntraj` trajectories (state in place, programs, readout
// (ntraj x T) or null, and optionally the state before every exponential:
// states[((b*T*F + n)*K + e)*M + row], rows in the layout's order).
int parts_forward_launch(sss_plan* p, const PartsForward& fw, int ntraj, double* d_state,
                         const double* d_prog, double t0, int T, double* d_readout,
                         double* d_states, cudaStream_t st);
}  // namespace sss
