// Bank-aware placement for the slot-programmed kernels (host code, used by
// sss_batch.cu).
//
// A warp's 64-bit shared-memory access is served per half-warp, one word
// per bank (word index mod 16) per wavefront: an instruction whose
// half-warp touches k distinct words in its fullest bank takes k
// wavefronts, and its lanes wait for them.  The slot program fixes the
// pieces each lane computes, but two things are free: the numbers of the
// rows and of the parked partial sums (labels), and the order of the items
// inside a piece (the terms of a sum).  optimise_banks() chooses both to
// minimise the extra wavefronts of one Horner term: simulated annealing
// over swaps of two labels of one class and of two items of one piece,
// three in four of them aimed at an access in the fullest bank of a
// conflicting instruction, keeping the best placement seen.
#pragma once
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

namespace sss {

// What one lane touches in one access instruction: the buffer (its base is
// a multiple of 16 words, so only the word index sets the bank; -1: no
// access) and the item (a row, a fixed row or a partial sum), whose word
// index is pos[item].
struct BankAccess {
    int buf, item;
};

// The accesses of one Horner term on an instruction x lane grid:
// cell[i*L + l] is lane l's access in instruction i; a half-warp is 16
// consecutive lanes (all L when L < 16).
struct BankProblem {
    int n_instr = 0, L = 0;
    std::vector<BankAccess> cell;
    std::vector<std::vector<int>> cell_sets;  // cells (of one lane) whose contents may be permuted
    std::vector<std::vector<int>> classes;    // items whose labels may be exchanged
};

namespace bank_detail {

// Extra wavefronts of instruction i on half-warp h: the distinct (buffer,
// word) pairs in its fullest bank, minus one.  (This reproduces the
// shared-memory conflict counts ncu reports for these kernels.)
inline int group_cost(const BankProblem& pb, int i, int h, const std::vector<int>& pos) {
    const int hw = pb.L < 16 ? pb.L : 16;
    int keys[16];
    int n = 0;
    for (int p = h * hw; p < (h + 1) * hw; p++) {
        const BankAccess& a = pb.cell[(size_t)i * pb.L + p];
        if (a.buf < 0) continue;
        const int k = a.buf * 65536 + pos[a.item];
        bool seen = false;
        for (int j = 0; j < n && !seen; j++) seen = keys[j] == k;
        if (!seen) keys[n++] = k;
    }
    int cnt[16] = {0};
    int most = 0;
    for (int j = 0; j < n; j++) {
        const int c = ++cnt[(keys[j] & 65535) & 15];
        if (c > most) most = c;
    }
    return most > 1 ? most - 1 : 0;
}

}  // namespace bank_detail

inline int bank_total_cost(const BankProblem& pb, const std::vector<int>& pos) {
    const int hw = pb.L < 16 ? pb.L : 16;
    int c = 0;
    for (int i = 0; i < pb.n_instr; i++)
        for (int h = 0; h < pb.L / hw; h++) c += bank_detail::group_cost(pb, i, h, pos);
    return c;
}

// Optimises pos (item -> word index, initially the labels) and the cell
// contents in place; origin[c] (output) is the cell whose original content
// cell c now holds.  Returns the extra wavefronts after, *before those
// before.  Deterministic (fixed seed); `budget` bounds the work in group
// evaluations.
inline int optimise_banks(BankProblem& pb, std::vector<int>& pos, std::vector<int>& origin,
                          long budget, int* before) {
    const int L = pb.L, n_items = (int)pos.size(), n_cells = (int)pb.cell.size();
    const int hw = L < 16 ? L : 16, n_half = L / hw;
    origin.resize(n_cells);
    for (int c = 0; c < n_cells; c++) origin[c] = c;
    std::vector<std::vector<int>> item_cells(n_items);
    for (int c = 0; c < n_cells; c++)
        if (pb.cell[c].buf >= 0) item_cells[pb.cell[c].item].push_back(c);
    std::vector<int> class_of(n_items, -1), set_of(n_cells, -1);
    for (int ci = 0; ci < (int)pb.classes.size(); ci++)
        if (pb.classes[ci].size() >= 2)
            for (int x : pb.classes[ci]) class_of[x] = ci;
    for (int si = 0; si < (int)pb.cell_sets.size(); si++)
        if (pb.cell_sets[si].size() >= 2)
            for (int c : pb.cell_sets[si]) set_of[c] = si;
    const int n_groups = pb.n_instr * n_half;
    std::vector<int> gcost(n_groups);
    int cost = 0;
    for (int g = 0; g < n_groups; g++) {
        gcost[g] = bank_detail::group_cost(pb, g / n_half, g % n_half, pos);
        cost += gcost[g];
    }
    if (before) *before = cost;
    long n_labels = 0, n_set_cells = 0;
    for (const auto& cl : pb.classes)
        if (cl.size() >= 2) n_labels += (long)cl.size();
    for (const auto& cs : pb.cell_sets)
        if (cs.size() >= 2) n_set_cells += (long)cs.size();
    const long n_moves = n_labels + n_set_cells;
    if (cost == 0 || n_moves == 0) return cost;
    std::vector<int> best_pos = pos, best_origin = origin;
    std::vector<BankAccess> best_cell = pb.cell;
    int best_cost = cost;
    std::vector<int> stamp((size_t)n_groups, -1), touched;
    std::mt19937 rng(20260311u);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    auto pick = [&](const std::vector<std::vector<int>>& sets, long total, int* set_out) {
        long r = (long)(uni(rng) * total);
        if (r >= total) r = total - 1;
        int si = 0;
        while (true) {
            const long sz = sets[si].size() >= 2 ? (long)sets[si].size() : 0;
            if (r < sz) break;
            r -= sz;
            si++;
        }
        *set_out = si;
        return (int)r;
    };
    auto touch_cell = [&](int c, long it) {
        const int i = c / L, h = (c % L) / hw;
        const int g = i * n_half + h;
        if (stamp[g] != (int)it) {
            stamp[g] = (int)it;
            touched.push_back(g);
        }
    };
    std::vector<int> newc;
    auto eval = [&](bool after) {
        int s = 0;
        if (after) newc.clear();
        for (int g : touched) {
            const int v = after ? bank_detail::group_cost(pb, g / n_half, g % n_half, pos) : gcost[g];
            if (after) newc.push_back(v);
            s += v;
        }
        return s;
    };
    // a cell in the fullest bank of a conflicting group (or -1): focuses
    // most moves on the accesses that cost wavefronts
    auto conflicting_cell = [&]() {
        for (int tries = 0; tries < 64; tries++) {
            const int g = (int)(uni(rng) * n_groups) % n_groups;
            if (gcost[g] == 0) continue;
            const int i = g / n_half, h = g % n_half;
            int cnt[16] = {0}, keys[16], kc[16], n = 0;
            for (int p = h * hw; p < (h + 1) * hw; p++) {
                const int c = i * L + p;
                const BankAccess& a = pb.cell[c];
                if (a.buf < 0) continue;
                const int k = a.buf * 65536 + pos[a.item];
                bool seen = false;
                for (int j = 0; j < n && !seen; j++) seen = keys[j] == k;
                if (!seen) {
                    keys[n] = k;
                    kc[n++] = c;
                    cnt[pos[a.item] & 15]++;
                }
            }
            int most = 0, bank = 0;
            for (int b = 0; b < 16; b++)
                if (cnt[b] > most) { most = cnt[b]; bank = b; }
            int pickc[16], m = 0;
            for (int j = 0; j < n; j++)
                if (((keys[j] & 65535) & 15) == bank) pickc[m++] = kc[j];
            if (m) return pickc[(int)(uni(rng) * m) % m];
        }
        return -1;
    };
    // the temperature falls geometrically from 0.3 to 0.05 extra wavefronts;
    // the search stops early once a third of the budget passes without a
    // new best
    long spent = 0, spent_at_best = 0;
    const long max_iters = budget / 4 + 1;
    for (long it = 0; spent < budget && it < max_iters && best_cost > 0 &&
                      spent - spent_at_best <= budget / 3;
         it++) {
        const double temp = 0.3 * std::pow(0.05 / 0.3, (double)spent / (double)budget);
        const double u = uni(rng) * (double)n_moves;
        int kind = u < (double)n_labels ? 0 : 1;
        touched.clear();
        int a = -1, b = -1;
        const int fc = uni(rng) < 0.75 ? conflicting_cell() : -1;
        if (fc >= 0) {
            // move the item of a conflicting cell: its label, or its place
            // in its piece
            const int item = pb.cell[fc].item;
            const bool can_label = class_of[item] >= 0, can_set = set_of[fc] >= 0;
            if (!can_label && !can_set) continue;
            kind = (can_label && (!can_set || uni(rng) < 0.5)) ? 0 : 1;
            if (kind == 0) {
                const auto& cl = pb.classes[class_of[item]];
                a = item;
                b = cl[(size_t)(uni(rng) * cl.size()) % cl.size()];
                if (a == b) continue;
                for (int x : {a, b})
                    for (int c : item_cells[x]) touch_cell(c, it);
            } else {
                const auto& cs = pb.cell_sets[set_of[fc]];
                a = fc;
                b = cs[(size_t)(uni(rng) * cs.size()) % cs.size()];
                if (a == b || (pb.cell[a].buf == pb.cell[b].buf && pb.cell[a].item == pb.cell[b].item))
                    continue;
                touch_cell(a, it);
                touch_cell(b, it);
            }
        } else if (kind == 0) {  // two labels
            int ci = 0;
            const int r = pick(pb.classes, n_labels, &ci);
            const auto& cl = pb.classes[ci];
            a = cl[(size_t)r];
            b = cl[(size_t)(uni(rng) * cl.size()) % cl.size()];
            if (a == b) continue;
            for (int x : {a, b})
                for (int c : item_cells[x]) touch_cell(c, it);
        } else {  // two items of one piece
            int si = 0;
            const int r = pick(pb.cell_sets, n_set_cells, &si);
            const auto& cs = pb.cell_sets[si];
            a = cs[(size_t)r];
            b = cs[(size_t)(uni(rng) * cs.size()) % cs.size()];
            if (a == b || (pb.cell[a].buf == pb.cell[b].buf && pb.cell[a].item == pb.cell[b].item))
                continue;
            touch_cell(a, it);
            touch_cell(b, it);
        }
        const int c0 = eval(false);
        auto apply = [&]() {
            if (kind == 0) std::swap(pos[a], pos[b]);
            else std::swap(pb.cell[a], pb.cell[b]);
        };
        apply();
        const int c1 = eval(true);
        spent += (long)touched.size();
        const int delta = c1 - c0;
        if (delta <= 0 || uni(rng) < std::exp(-delta / temp)) {
            if (kind == 1) {
                // cells a and b exchanged contents: update the item lists
                if (pb.cell[a].buf >= 0)
                    for (int& c : item_cells[pb.cell[a].item])
                        if (c == b) { c = a; break; }
                if (pb.cell[b].buf >= 0)
                    for (int& c : item_cells[pb.cell[b].item])
                        if (c == a) { c = b; break; }
                std::swap(origin[a], origin[b]);
            }
            for (size_t k = 0; k < touched.size(); k++) gcost[touched[k]] = newc[k];
            cost += delta;
            if (cost < best_cost) {
                best_cost = cost;
                best_pos = pos;
                best_cell = pb.cell;
                best_origin = origin;
                spent_at_best = spent;
            }
        } else {
            apply();  // every move is its own inverse
        }
    }
    pos = best_pos;
    pb.cell = best_cell;
    origin = best_origin;
    return best_cost;
}

}  // namespace sss
