// Arguments of the batched forward kernels and their launch helper, shared
// by the translation units that hold those kernels (sss_batch.cu: row-part,
// register and shared-memory variants; sss_slots_warp.cu, sss_slots_cta.cu
// and sss_phased.cu: the slot-packed and phased row-part variants).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "sss_internal.cuh"

namespace sss {

constexpr int kMaxTaylor = 24;

struct BatchArgs {
    int M;        // state rows kept (reachable)
    int Ga;       // active generators
    int K, Q, F, nch, nseg, T_max, ntraj, degree, substeps, N;
    int E;        // entries per lane (max over lanes)
    int t_begin, t_end;        // output samples of this launch
    double h_sub, t0, dt;
    int gen_index[kMaxSlots];  // active generator -> coefficient slot
    const double* toff;        // F: (r*dt)/F
    const double* noff;        // Q: (dt*node_k)/F
    const double* W;           // K*Q
    const double* gv;          // Ga * E * L  generator values [g][e][l]
    const unsigned* ent;       // E * L  packed entry words [e][l]
    const int* lane_rows;      // L: entries of each lane
    const int* rbeg;           // L+1: rows [rbeg[l], rbeg[l+1]) belong to lane l
    const int* row_orig;       // M
    const double* rw;          // M readout weights (or null)
    const double* rho0;        // ntraj*N  state at sample t_begin
    const double* prog;        // ntraj*nch*nseg*5
    const int* samples;        // ntraj or null
    double* readout;           // ntraj*T_max or null
    double* fin;               // ntraj*N  state after the launch (may alias rho0), or null
    double* trace;             // ntraj*T_max*N  state after every output sample, or null
    int* queue;
    // row-part variant
    const int* pcol;           // C*P*L  column of each part entry [e][l] (M: the zero row)
    const unsigned* cw;        // kCloseMax*L  close words [k][l]
    const double* om0;         // K*C*P*L  constant part of Omega per exponential
    int kc;                    // close slots per lane (max over lanes)
    int n_live;                // generators assembled per step (the others are in om0)
    int live[kMaxSlots];       // their active-generator slots
    int live_k[kMaxSlots];     // node of a rotating slot (weight W[e,k] c_k), -1: sum over nodes
    int live_ch[kMaxSlots];    // index of its channel among the live channels
    int n_lch;                 // live channels (sampled into the ring)
    int lch_chan[kMaxSlots];   // their program channel (>= nch: zero)
    // generalised rotating frame (state in the eigenbasis of L0)
    int rot, resid;
    const double* Vm;          // N*N eigenvectors (lab = V x)
    const double* Vinvm;       // N*N inverse (x = V^-1 rho)
    const double* blk_self;    // M: e^{L0 h} diagonal coefficient of each row (minus 1 when residual)
    const double* blk_part;    // M: coefficient of its partner row
    const int* blk_pos;        // M: the partner's row (M: none, the zero row)
    const int* order;          // ntraj: queue position -> trajectory (longest first), or null
    // coefficient table instead of programs (row-part kernel): per trajectory
    // F*T_max*Q rows of tab_G values, row (r*T_max + t)*Q + k for node k of
    // fine step r of output sample t; a slot's channel is its table column
    const double* tab;
    int tab_G;
    double* states;            // state before every exponential, or null:
    long st_steps;             //   [((b*st_steps + n)*K + e)*M + row], n = step since t_begin
    double inv_j[kMaxTaylor + 1];
    // slot-packed and phased row-part variants (kernel slot words in cw;
    // om0 and gv [.][q][l])
    int S;                     // slots per lane
    int bar_at;                // barrier slot
    int npart;                 // parked partial sums per trajectory
    unsigned amask[kMaxSlots]; // per live generator: slots with a non-zero value in some lane
    double cfac[kMaxTaylor + 1];  // scaled Horner: c_j = d!/(j-1)!
    double inv_dfact;          // 1/d!
    // health word of the run, or null: all ones while every readout and
    // final-state entry written so far is finite, else the smallest
    // (output sample << 32 | trajectory) that was not
    unsigned long long* health;
};

// Records a non-finite readout or final-state entry x of trajectory b at
// output sample t (a final state counts as sample t_end) in the health word.
// One compare per written value; the atomic runs only on the error path.
__device__ __forceinline__ void note_nonfinite(const BatchArgs& a, double x, int b, int t) {
    if (!isfinite(x) && a.health)
        atomicMin(a.health, ((unsigned long long)(unsigned)t << 32) | (unsigned)b);
}

// Slot words.
// Logical words (the packer's, and sss_slot_layout's): bits 0-13 the row an
// entry reads or a close closes, or the partial index of a partial add; bit
// 14 partial add; bit 15 close; bit 16 piece start; bit 17 start from
// partial pidx; bit 18 park the sum as partial pidx; bits 19-31 pidx.
constexpr unsigned kSlotIdx = 0x3fffu, kSlotPart = 1u << 14, kSlotClose = 1u << 15,
                   kSlotStart = 1u << 16, kSlotRecv = 1u << 17, kSlotDend = 1u << 18;
constexpr int kSlotPidxShift = 19;
// Kernel words: per slot a load word (bits 0-13 offset, bits 14-15 source:
// 0 current iterate, 1 v, 2 the next iterate's partial area) and a store
// word (bits 0-13 store offset in the next iterate, bits 14-27 start-value
// offset there -- the zero row or a partial sum --, bit 28 piece start).
constexpr unsigned kLdV = 1u << 14, kLdNext = 2u << 14, kStStart = 1u << 28;
// Slot counts with a compiled slot-packed kernel (the packer takes the
// smallest that fits).
constexpr int kSlotSizes[] = {4, 5, 6, 7, 8, 10, 12, 14, 16};
inline bool slot_size_compiled(int S) {
    for (int s : kSlotSizes)
        if (s == S) return true;
    return false;
}
// Shapes of the phased row-part kernel: per lane C1 chains of P1 slots in
// phase 1, then C2 chains of P2 slots in phase 2 (slots per lane
// C1*P1 + C2*P2), in increasing order of slots.
struct PhasedShape {
    int C1, P1, C2, P2;
};
constexpr PhasedShape kPhasedShapes[] = {{1, 3, 1, 1}, {1, 4, 1, 1}, {1, 4, 1, 2}, {2, 3, 1, 1},
                                         {2, 4, 1, 1}, {2, 4, 1, 2}, {4, 4, 2, 1}, {4, 4, 2, 2}};
constexpr int kPhasedShapeCount = (int)(sizeof(kPhasedShapes) / sizeof(kPhasedShapes[0]));

// Launch a persistent batched kernel: one group per trajectory with work in
// this launch, at most what fits on the GPU at once.
template <class Kern>
inline int launch(sss_plan* p, Kern kern, const BatchArgs& a, int threads, int slots_per_cta,
           size_t smem, cudaStream_t st) {
    SSS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    SSS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
    if (per_sm < 1) return fail(SSS_EINVAL, "batched kernel does not fit on an SM");
    // one group per trajectory with work in this launch (at most as many as
    // fit): every group then starts on a trajectory of its own and the CTAs
    // spread evenly over the SMs (a grid sized for trajectories that only
    // pad their readout would leave the working ones wherever the queue
    // happened to hand them out)
    const int n_work = p->launch_active > 0 ? std::min(p->launch_active, a.ntraj) : a.ntraj;
    int want = (n_work + slots_per_cta - 1) / slots_per_cta;
    int grid = std::max(1, std::min(want, per_sm * p->num_sms));
    // the launch's own timing events, except while the stream is being
    // captured into a graph (events recorded there cannot be waited on)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    SSS_CUDA(cudaStreamIsCapturing(st, &cap));
    const bool timed = cap == cudaStreamCaptureStatusNone;
    if (timed && !p->ev_begin) {
        SSS_CUDA(cudaEventCreate(&p->ev_begin));
        SSS_CUDA(cudaEventCreate(&p->ev_end));
    }
    if (timed && !p->ev_keep_begin) SSS_CUDA(cudaEventRecord(p->ev_begin, st));
    kern<<<grid, threads, smem, st>>>(a);
    SSS_CUDA(cudaGetLastError());
    if (timed) {
        SSS_CUDA(cudaEventRecord(p->ev_end, st));
        p->ev_recorded = true;
    }
    p->last_grid = grid;
    return SSS_OK;
}

// The slot-packed kernel for L lanes and S slots (sss_slots_warp.cu for
// L <= 32, sss_slots_cta.cu for wider groups), and the phased row-part
// kernel for L lanes (8, 16 or 32) and kPhasedShapes[shape] (sss_phased.cu).
int launch_slots_warp(sss_plan* p, int L, int S, const BatchArgs& a, int threads, size_t smem,
                      cudaStream_t st);
int launch_slots_cta(sss_plan* p, int L, int S, const BatchArgs& a, int threads, size_t smem,
                     cudaStream_t st);
int launch_phased(sss_plan* p, int L, int shape, const BatchArgs& a, int threads, size_t smem,
                  cudaStream_t st);
inline int launch_slots(sss_plan* p, int L, int S, const BatchArgs& a, int threads, size_t smem,
                        cudaStream_t st) {
    return L <= 32 ? launch_slots_warp(p, L, S, a, threads, smem, st)
                   : launch_slots_cta(p, L, S, a, threads, smem, st);
}

}  // namespace sss
