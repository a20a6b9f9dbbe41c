// The automatic lane count of the batched kernels and the lane-count phases
// of a batch of uneven lengths (host code, used by sss_batch.cu).
//
// A layout at L lanes per trajectory issues cost FP64 warp-instructions per
// trajectory and Horner term (cost[i] for L = 8 << i, 0 where nothing fits);
// n trajectories make ceil(n L / 32) warps over the GPU's SM
// sub-partitions (four per SM), and the busiest sub-partition issues
// ceil(warps / sub-partitions) x cost per term.  The rule takes the lane
// count with the smallest such figure.  On a tie the narrower group wins once
// its warps fill every sub-partition -- the same issue count with fewer group
// barriers and shuffles per instruction -- and the wider one wins before
// that, where more warps hide more latency.
//
// An uneven batch loses trajectories as it runs, and the rule asks for
// wider groups as fewer remain.  The batch runs in phases, each at one lane
// count, each wider than the last: a phase ends at the first output sample
// after which the rule, for the trajectories still running, asks for more
// lanes than the phase has.  Where the rule drops back to a narrower count
// on a tie, the phase runs on.
#pragma once
#include <algorithm>
#include <functional>
#include <vector>

namespace sss {

constexpr int kLaneCounts = 6;  // lanes per trajectory 8, 16, ..., 256 of the row kernels

// lanes per trajectory for n trajectories on `subparts` SM sub-partitions
// (0: no lane count fits)
inline int auto_lane_count(long subparts, const double* cost, long n) {
    int best = 0;
    double best_v = 0.0;
    long best_warps = 0;
    for (int i = 0; i < kLaneCounts; i++) {
        if (cost[i] <= 0.0) continue;
        const long Lc = 8L << i;
        const long warps = (std::max(1L, n) * Lc + 31) / 32;
        const double v = (double)((warps + subparts - 1) / subparts) * cost[i];
        if (!best || v < best_v || (v == best_v && best_warps < subparts)) {
            best = (int)Lc;
            best_v = v;
            best_warps = warps;
        }
    }
    return best;
}

// trajectories with more than t output samples, from the sample counts
// sorted longest first
inline int running_after(const std::vector<int>& longest, int t) {
    return (int)(std::lower_bound(longest.begin(), longest.end(), t, std::greater<int>()) -
                 longest.begin());
}

// the running count, below n_now, at which a phase of L lanes ends: the
// largest n < n_now for which the rule asks for more than L lanes (-1: the
// phase runs to the end)
inline int phase_end_count(long subparts, const double* cost, int L, int n_now) {
    for (int n = n_now - 1; n >= 1; n--)
        if (auto_lane_count(subparts, cost, n) > L) return n;
    return -1;
}

}  // namespace sss
