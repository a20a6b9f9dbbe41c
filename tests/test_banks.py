"""The bank-aware placement of the slot-programmed kernels (host code,
superspinsim_gb300/csrc/sss_banks.h), compiled with g++ into a small test
program: the conflict model on hand-made accesses; the annealer keeps
labels a permutation within their class, moves cell contents only within
their sets, reports costs consistent with the model, and removes conflicts
that relabelling or reordering can remove.  No GPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

PROGRAM = r'''
#include "sss_banks.h"
#include <algorithm>
#include <cstdio>
using namespace sss;

static int fails = 0;
#define CHECK(c) do { if (!(c)) { std::printf("FAIL line %d: %s\n", __LINE__, #c); fails++; } } while (0)

static std::vector<int> identity(int n) {
    std::vector<int> v(n);
    for (int i = 0; i < n; i++) v[i] = i;
    return v;
}

int main() {
    // the conflict model: one instruction, one half-warp of 16 lanes
    {
        BankProblem pb;
        pb.n_instr = 1;
        pb.L = 16;
        const std::vector<int> pos = identity(64);
        for (int l = 0; l < 16; l++) pb.cell.push_back({1, l});  // words 0..15, one per bank
        CHECK(bank_total_cost(pb, pos) == 0);
        pb.cell[3] = {1, 0};   // the same word again: a broadcast
        CHECK(bank_total_cost(pb, pos) == 0);
        pb.cell[3] = {1, 16};  // word 16 shares bank 0 with word 0
        CHECK(bank_total_cost(pb, pos) == 1);
        pb.cell[4] = {1, 32};  // a third word in bank 0
        CHECK(bank_total_cost(pb, pos) == 2);
        pb.cell[5] = {2, 0};   // word 0 of another buffer: a fourth
        CHECK(bank_total_cost(pb, pos) == 3);
        pb.cell[6] = {-1, 0};  // no access
        CHECK(bank_total_cost(pb, pos) == 3);
    }
    // labels only: 32 lanes x 8 instructions; lane l reads row (16 l + i)
    // mod 48 in instruction i, so each half-warp reads rows i, 16 + i and
    // 32 + i, all in bank i under the identity numbering
    {
        BankProblem pb;
        pb.n_instr = 8;
        pb.L = 32;
        const int M = 48;
        for (int i = 0; i < 8; i++)
            for (int l = 0; l < 32; l++) pb.cell.push_back({1, (l * 16 + i) % M});
        pb.classes.push_back(identity(M));
        std::vector<int> pos = identity(M), origin;
        const int start = bank_total_cost(pb, pos);
        int before = -1;
        const int after = optimise_banks(pb, pos, origin, 2000000, &before);
        CHECK(before == start);
        CHECK(after == bank_total_cost(pb, pos));
        CHECK(before == 32 && after == 0);
        std::vector<int> sorted_pos(pos);
        std::sort(sorted_pos.begin(), sorted_pos.end());
        CHECK(sorted_pos == identity(M));
        for (size_t c = 0; c < pb.cell.size(); c++) CHECK(origin[c] == (int)c);
        std::printf("labels %d -> %d\n", before, after);
    }
    // items only (no label may move): lane l reads rows l%8 and l%8 + 16,
    // which share a bank, in instructions 0 and 1 -- lanes 0..7 in one order,
    // lanes 8..15 in the other, so every instruction mixes the two halves.
    // Reordering each lane's two items (its set) removes every conflict.
    {
        BankProblem pb;
        pb.n_instr = 2;
        pb.L = 16;
        for (int i = 0; i < 2; i++)
            for (int l = 0; l < 16; l++) {
                const bool low_first = (i == 0) == (l < 8);
                pb.cell.push_back({1, low_first ? l % 8 : l % 8 + 16});
            }
        for (int l = 0; l < 16; l++) pb.cell_sets.push_back({l, 16 + l});
        std::vector<int> pos = identity(24), origin;
        const std::vector<BankAccess> cells0 = pb.cell;
        int before = -1;
        const int after = optimise_banks(pb, pos, origin, 200000, &before);
        CHECK(before > 0);
        CHECK(after == 0);
        CHECK(pos == identity(24));
        for (size_t c = 0; c < pb.cell.size(); c++) {
            const int o = origin[c];
            CHECK(o % 16 == (int)c % 16);  // stays in its lane
            CHECK(pb.cell[c].item == cells0[o].item && pb.cell[c].buf == cells0[o].buf);
        }
        std::printf("items %d -> %d\n", before, after);
    }
    return fails;
}
'''


def test_bank_placement_program():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    build = os.path.join(ROOT, "tests", "_build")
    os.makedirs(build, exist_ok=True)
    src = os.path.join(build, "banks_test.cpp")
    exe = os.path.join(build, "banks_test")
    with open(src, "w") as f:
        f.write(PROGRAM)
    inc = os.path.join(ROOT, "superspinsim_gb300", "csrc")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", inc, src, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and "FAIL" not in out.stdout, out.stdout + out.stderr
