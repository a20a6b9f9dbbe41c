"""The slot-packed layout of the batched kernel (sss_slot_layout, host only):
every lane runs the same S FMA slots per Horner term w <- v + (Omega w)/j.
These tests emulate one Horner term slot by slot from the layout's slot
words, with the one barrier between the donor and receiver phases, and
compare it with the direct sparse product: every entry used once, every
row closed once, no partial sum read before the barrier or before it was
parked, and the result equal to v + (A x)/j.  No GPU needed."""
import numpy as np
import pytest

from conftest import load_case

IDX, PART, CLOSE, START, RECV, DEND, PSHIFT = 0x3fff, 1 << 14, 1 << 15, 1 << 16, 1 << 17, 1 << 18, 19


def _csr(rows):
    row_ptr = np.zeros(len(rows) + 1, dtype=np.int32)
    row_ptr[1:] = np.cumsum([len(r) for r in rows])
    col = np.array([c for r in rows for c in r], dtype=np.int32)
    return row_ptr, col


def _emulate(M, col, vals, x, v, ij, S, bar, npart, words, entries):
    """One Horner term of the slot program; returns next (M,)."""
    L = words.shape[1]
    part = np.zeros(npart + 1)
    written = np.zeros(npart + 1, dtype=bool)
    nxt = np.full(M, np.nan)
    closed = np.zeros(M, dtype=int)
    used = np.zeros(col.size, dtype=int)
    xs = np.append(x, 0.0)  # the zero row M
    vs = np.append(v, 0.0)
    s = np.zeros(L)
    for lo, hi in ((0, bar), (bar, S)):
        for ln in range(L):
            for q in range(lo, hi):
                w = int(words[q, ln])
                e = int(entries[q, ln])
                idx, pidx = w & IDX, w >> PSHIFT
                pre = (vs if w & CLOSE else xs)[M if w & PART else idx]
                if w & RECV or w & PART:
                    assert q >= bar, "a partial sum read before the barrier"
                    assert written[pidx if w & RECV else idx], "a partial sum read before it was parked"
                xin = part[idx] if w & PART else pre
                base = ((part[pidx] if w & RECV else 0.0) if w & START else s[ln])
                if w & CLOSE:
                    s[ln] = base*ij + xin
                    nxt[idx] = s[ln]
                    closed[idx] += 1
                else:
                    coef = 1.0 if e == -2 else (vals[e] if e >= 0 else 0.0)
                    if e >= 0:
                        used[e] += 1
                        assert idx == col[e]
                    s[ln] = coef*xin + base
                if w & DEND:
                    assert q < bar, "a partial sum parked after the barrier"
                    part[pidx] = s[ln]
                    written[pidx] = True
    assert np.all(closed == 1), "every row closed exactly once"
    assert np.all(used == 1), "every entry used exactly once"
    return nxt


def _check(rows, lanes, seed=0, expect_slots=None):
    from superspinsim_gb300 import _lib
    M = len(rows)
    row_ptr, col = _csr(rows)
    S, bar, npart, words, entries = _lib.slot_layout(row_ptr, col, lanes)
    assert S >= -(-int(col.size + M)//lanes)
    if expect_slots is not None:
        assert S == expect_slots
    rng = np.random.default_rng(seed)
    vals = rng.standard_normal(col.size)
    x, v = rng.standard_normal(M), rng.standard_normal(M)
    ij = 1/7
    nxt = _emulate(M, col, vals, x, v, ij, S, bar, npart, words, entries)
    A = np.zeros((M, M))
    for i in range(M):
        for k in range(row_ptr[i], row_ptr[i + 1]):
            A[i, col[k]] += vals[k]
    ref = v + ij*(A @ x)
    assert np.abs(nxt - ref).max() <= 1e-13*max(1.0, np.abs(ref).max())
    return S, bar, npart


def _pruned_rows(gens, rho_flat, active):
    """Rows reachable from the support of rho_flat under the union pattern
    of the active generators, and each row's columns (compressed)."""
    N = gens.shape[1]
    U = np.zeros((N, N), dtype=bool)
    for g in active:
        U |= gens[g] != 0
    reach = set(np.nonzero(rho_flat)[0])
    stack = list(reach)
    while stack:
        c = stack.pop()
        for r in np.nonzero(U[:, c])[0]:
            if r not in reach:
                reach.add(int(r))
                stack.append(int(r))
    rows = sorted(reach)
    pos = {r: k for k, r in enumerate(rows)}
    return [[pos[c] for c in np.nonzero(U[r])[0] if c in pos] for r in rows]


def test_nv7_odmr_pattern_packs_to_seven_slots_at_16_lanes():
    """The headline workload's pattern (19 rows, 87 entries: 106 slot
    operations) fits 16 lanes x 7 slots (112) and 8 lanes x 14."""
    c = load_case("nv7_n49")
    gens, vm = c["generators"], c["vectorisation_map"]
    rho = np.zeros(vm.shape[0])
    rho[1] = 1.0
    rows = _pruned_rows(gens, rho, [0, 1, 4])
    assert len(rows) == 19 and sum(map(len, rows)) == 87
    assert _check(rows, 16, expect_slots=7)[0] == 7
    assert _check(rows, 8, expect_slots=14)[0] == 14
    _check(rows, 32)


@pytest.mark.parametrize("lanes", [128, 256])
def test_nv21_pattern(lanes):
    c = load_case("nv21_n441")
    gens, vm = c["generators"], c["vectorisation_map"]
    rho = np.zeros(vm.shape[0])
    for k, (y, x, ch) in enumerate(vm):
        if y == x and ch == 0 and y in (3, 4, 5):
            rho[k] = 1/3
    rows = _pruned_rows(gens, rho, [0, 1, 4])
    S, _, _ = _check(rows, lanes)
    assert S <= 16


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("lanes", [8, 16, 32, 64])
def test_random_patterns(seed, lanes):
    """Ragged rows (empty rows, rows longer than the slot count, repeated
    columns) on every lane count that can hold them."""
    rng = np.random.default_rng(1000*lanes + seed)
    M = int(rng.integers(1, 60))
    rows = []
    for _ in range(M):
        n = int(rng.choice([0, 1, 2, 3, 5, 8, 13, 20], p=[.1, .15, .2, .2, .15, .1, .06, .04]))
        rows.append(sorted(rng.integers(0, M, n).tolist()))
    from superspinsim_gb300 import _lib
    total = sum(map(len, rows)) + M
    if -(-total//lanes) > _lib.SLOTS_MAX:
        pytest.skip("pattern too large for this lane count")
    try:
        _check(rows, lanes, seed)
    except _lib.SSSError as e:
        # a pattern may not fit 16 slots at this lane count; the error says so
        assert e.code == -1 and "no slot layout" in str(e)


def test_empty_pattern_and_bad_arguments():
    from superspinsim_gb300 import _lib
    S, bar, npart, words, entries = _lib.slot_layout([0, 0, 0], [], 8)
    assert S == 4 and npart == 0  # the smallest compiled slot count
    assert np.count_nonzero(words & CLOSE) == 2
    with pytest.raises(_lib.SSSError):
        _lib.slot_layout([0, 1], [5], 8)  # column out of range
    with pytest.raises(_lib.SSSError):
        _lib.slot_layout([0, 0], [], 12)  # lanes not a power of two
