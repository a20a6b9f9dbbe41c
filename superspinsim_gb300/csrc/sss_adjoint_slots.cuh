// Arguments of the slot-programmed adjoint backward kernel (sss_adjoint_slots.cu),
// shared with its host set-up in sss_adjoint.cu.
//
// The backward sweep's series for one exponential is the Taylor action of
// the block matrix B = [[Omega^T, G^T], [0, Omega^T]] on [0; mu]: its top
// half is L(Omega^T, G^T) mu (so g = rho_before . px) and its bottom half
// E^T mu (the new adjoint).  That is a forward-style series on a matrix of
// 2M rows -- px rows hold Omega^T and G^T entries, py rows Omega^T entries
// and a v term -- so it runs on the slot programs of the forward kernels
// (scaled Horner, phased or slot-packed), with v = [0; mu]: the px rows' v
// terms read zeros.  G^T entries are constant entries (their values do not
// depend on the exponential's coefficients).
#pragma once
#include "sss_batch_args.cuh"

namespace sss {

struct AdjSlotArgs {
    int M;           // forward rows (compressed order)
    int M2;          // block rows, 2M (zero row M2, sink M2 + 1, partial sums after)
    int Ms;          // block buffer stride (a multiple of 16 words)
    int K, Q, F, nch, nseg, ntraj, degree, T;
    long n_steps;
    double h, t0, dt;
    int n_live, x_live, dch, npar;
    int live[kMaxG];          // live active-generator slots (their coefficient is assembled)
    int gen_index[kMaxG];     // active-generator slot -> generator
    unsigned amask[kMaxG];    // per live generator: the slots where some lane has a value
    const unsigned* cw;       // 2*S*L slot words
    const double* om0;        // K*S*L constant part of the block per exponential [e][q][l]
    const double* gv;         // Ga*S*L generator values [g][q][l]
    const int* ppx;           // M: block position of forward row i's px
    const int* ppy;           // M: ... and of its py
    const int* fpos;          // M: position of forward row i in the stored states
    const double* rw;         // M: readout weights
    const double* tw;         // T
    const double* toff;
    const double* noff;
    const double* W;
    const double* states;     // ntraj*n_steps*K*M
    const double* readout;    // ntraj*T
    const double* prog;
    double* J;
    double* grad;
    int* queue;
    double cfac[kMaxTaylor + 1];  // scaled Horner: c_j = d!/(j-1)!
    double inv_dfact;             // 1/d!
};

// Launch the backward kernel for a slot layout of the block matrix: phased
// row parts (shape) or slot-packed (S slots) at L lanes; SSS_EINVAL when no
// kernel is compiled for that layout.
int launch_adjoint_slots(sss_plan* p, int L, bool phased, int shape, int S, const AdjSlotArgs& a,
                         int threads, size_t smem, cudaStream_t st);

}  // namespace sss
