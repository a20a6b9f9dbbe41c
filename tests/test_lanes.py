"""The automatic lane count of the batched kernels and the phases of an
uneven batch (host code, superspinsim_gb300/csrc/sss_lanes.h), compiled with
g++ into a small test program: the busiest sub-partition's issue count
decides, ties go to the narrower group once its warps fill every
sub-partition and to the wider one before, and a phase ends only where the
rule asks for a wider group.  No GPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

PROGRAM = r'''
#include "sss_lanes.h"
#include <cstdio>
using namespace sss;

static int fails = 0;
#define CHECK(c) do { if (!(c)) { std::printf("FAIL line %d: %s\n", __LINE__, #c); fails++; } } while (0)

int main() {
    const long sp = 4 * 152;  // SM sub-partitions of a 152-SM GPU
    // FP64 instructions per trajectory and Horner term of the NV-7 Ramsey
    // layouts: 8 lanes 14 slots, 16 lanes 7, 32 lanes 6; nothing wider
    const double nv7[kLaneCounts] = {14, 7, 6, 0, 0, 0};
    // 4096: 8 lanes 2 x 14 = 28, 16 lanes 4 x 7 = 28 (tie, 1024 warps of
    // 8-lane groups fill 608 sub-partitions: the narrower), 32 lanes 7 x 6
    CHECK(auto_lane_count(sp, nv7, 4096) == 8);
    // 3648: 16 lanes 3 x 7 = 21 against 2 x 14
    CHECK(auto_lane_count(sp, nv7, 3648) == 16);
    CHECK(auto_lane_count(sp, nv7, 3649) == 8);
    // 2432: 608 warps of 8 lanes, 1 x 14 against 2 x 7 (tie, filled: 8)
    CHECK(auto_lane_count(sp, nv7, 2432) == 8);
    // 2000: 500 warps of 8 lanes leave sub-partitions empty: the tie goes wide
    CHECK(auto_lane_count(sp, nv7, 2000) == 16);
    // 608 and fewer: 32 lanes, 1 x 6 against 1 x 7
    CHECK(auto_lane_count(sp, nv7, 609) == 16);
    CHECK(auto_lane_count(sp, nv7, 608) == 32);
    CHECK(auto_lane_count(sp, nv7, 1) == 32);
    CHECK(auto_lane_count(sp, nv7, 0) == 32);  // counted as one trajectory
    // equal costs and few warps: the widest
    const double flat[kLaneCounts] = {4, 4, 4, 0, 0, 0};
    CHECK(auto_lane_count(sp, flat, 10) == 32);
    // equal costs once the narrowest fills every sub-partition: the wider
    // ones put more warps on the busiest
    CHECK(auto_lane_count(sp, flat, 2432) == 8);
    // a count that does not fit is skipped; nothing fits: 0
    const double only64[kLaneCounts] = {0, 0, 0, 3, 0, 0};
    CHECK(auto_lane_count(sp, only64, 1000) == 64);
    const double none[kLaneCounts] = {0, 0, 0, 0, 0, 0};
    CHECK(auto_lane_count(sp, none, 1000) == 0);

    // phases: 8 lanes from 4096 until 3648 run; 16 lanes until 608, past
    // the tie at 2432 where the rule would go back to 8 lanes; 32 to the end
    CHECK(phase_end_count(sp, nv7, 8, 4096) == 3648);
    CHECK(phase_end_count(sp, nv7, 16, 3648) == 608);
    CHECK(phase_end_count(sp, nv7, 32, 608) == -1);
    CHECK(phase_end_count(sp, nv7, 8, 1) == -1);

    // running counts from sample counts sorted longest first
    const std::vector<int> longest = {10, 7, 7, 3};
    CHECK(running_after(longest, 0) == 4);
    CHECK(running_after(longest, 3) == 3);
    CHECK(running_after(longest, 5) == 3);
    CHECK(running_after(longest, 7) == 1);
    CHECK(running_after(longest, 10) == 0);
    CHECK(running_after(std::vector<int>(), 0) == 0);
    return fails;
}
'''


def test_lane_rule_program():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    build = os.path.join(ROOT, "tests", "_build")
    os.makedirs(build, exist_ok=True)
    src = os.path.join(build, "lanes_test.cpp")
    exe = os.path.join(build, "lanes_test")
    with open(src, "w") as f:
        f.write(PROGRAM)
    inc = os.path.join(ROOT, "superspinsim_gb300", "csrc")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", inc, src, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and "FAIL" not in out.stdout, out.stdout + out.stderr
