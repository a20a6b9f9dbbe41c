"""Spin-system description -> real Hermitian-basis Lindblad generators.

Host-side set-up that runs once per model, restating the reference's
``superspinsim/generate_generators.py`` (``generate_atoms`` :19-166 and its
helpers) with complex matrices and vectorised superoperator construction.
It keeps the reference's conventions, because the generators and the state
layout are the interface of the time-stepping core:

* magnetic numbers run +S ... -S (:974-977); within an atom the nucleus is
  the faster index, and within a block later atoms are faster
  (:1017-1068, kron order of ``_kronecker_product`` :1071-1099);
* when a spin joins a block, jump operators are split per basis state of
  the other factor (``_kronecker_jump_inner/outer`` :1102-1157) and empty
  pieces dropped;
* all non-jump, non-projector operators of the atoms are made traceless
  (:752-767);
* blocks are direct-summed (:1300-1434); the ``allowed`` mask keeps the
  in-block entries (all entries without ``use_incoherent``);
* the Hermitian basis lists the allowed diagonal entries first, then the
  allowed upper pairs (y < x) as (re, im) (``_generate_valid_indices``
  :2361-2382); superoperators are -i[H, rho] (:2100-2160) and
  L rho L^+ - {L^+ L, rho}/2 (:2163-2223) in that basis;
* superoperators are grouped by label into L0 = H0 + D + Vc, Gx, Gy, Gz
  and Gr (:2226-2314), including the reference's exact-label rule that
  keeps a dephasing operator in D only while it is unsplit.

Physical models supported: electron spin with zero-field splitting, g
tensor (isotropic/axial), bias field, Lindblad dephasing (TS2) and
Boltzmann thermalisation (TS1); nucleus with quadrupole, nuclear g,
dephasing and thermalisation; hyperfine coupling; spin-spin (J) coupling
within a block; the NV inter-block couplings (spin-conserving and
non-conserving optical excitation/decay, intersystem crossing both ways);
the hBN-style Bell-state couplings between a singlet and a pair of
spin-1/2 atoms; and coherent (Hamiltonian) couplings between blocks,
constant or scaled by the fourth control channel, whose blocks' mutual
coherences join the allowed set through the transitive closure of the
coupling graph.
"""
import copy
import math

import numpy as np

from superspinsim_gb300 import params as default_params

JUMP_PREFIXES = ("LS1", "LI1", "Lrc", "Llc", "Lrn", "Lln", "Lisc", "Lbell", "Vr", "Vc")
GROUPS = {"D": ("LS1", "LI1", "LS2", "LI2", "Llc", "Lln", "Lisc", "Lbell"),
          "Gr": ("Lrc", "Lrn", "Vr"), "Vc": ("Vc",)}


# ---------------------------------------------------------------------------
# single spins
# ---------------------------------------------------------------------------

def spin_matrices(spin):
    """(Sx, Sy, Sz) on the basis m = +S ... -S, and the projector of each m
    keyed by its label."""
    dim = int(round(2*spin + 1))
    if dim == 1:
        z = np.zeros((1, 1), complex)
        return (z, z.copy(), z.copy()), {_proj_key(spin, 0): np.ones((1, 1), complex)}
    m = np.linspace(spin, -spin, dim)
    up = np.sqrt((spin - m)*(1 + spin + m))[1:]
    down = np.sqrt((spin + m)*(1 + spin - m))[:-1]
    sp = np.diag(up, 1)
    sm = np.diag(down, -1)
    sx = ((sp + sm)/2).astype(complex)
    sy = (1j*(sm - sp)/2)
    sz = np.diag(m).astype(complex)
    proj = {}
    for idx in range(dim):
        p = np.zeros((dim, dim), complex)
        p[idx, idx] = 1
        proj[_proj_key(spin, m[idx])] = p
    return (sx, sy, sz), proj


def _num(spin, m):
    m = 0.0 if abs(m) < 1e-12 else m
    return f"{m:.0f}" if abs(math.fmod(spin, 1)) < 1e-9 else f"{m:.1f}"


def _proj_key(spin, m):
    n = _num(spin, m)
    return f"|{n})({n}|"


def _axial(iso, tensor_kind, atom, prefix):
    """diag(iso - dip, iso - dip, iso + 2 dip) from iso/perp/dipole keys."""
    if prefix in atom:
        g = atom[prefix]
        if f"{prefix}_dipole" in atom:
            dip = atom[f"{prefix}_dipole"]
        elif f"{prefix}_perp" in atom:
            dip = (g - atom[f"{prefix}_perp"])/3
            g -= 2*dip
        else:
            dip = 0.0
    else:
        g, dip = iso, 0.0
    return np.diag([g - dip, g - dip, g + 2*dip]).astype(float)


def _quad(tensor, left, right):
    out = np.zeros_like(left[0])
    for i in range(3):
        for j in range(3):
            if tensor[i, j] != 0:
                out = out + tensor[i, j]*(left[i] @ right[j])
    return out


def _lin(tensor, vec):
    return tuple(sum(tensor[i, j]*vec[j] for j in range(3)) for i in range(3))


def _zfs_tensor(longitudinal, transverse):
    return np.diag([transverse - longitudinal/3, -transverse - longitudinal/3,
                    2*longitudinal/3])


def _thermal_jumps(prefix, quiescent, atom, T1, P):
    """Boltzmann thermalisation jumps sqrt(b_f/((b_i + b_f) T1)) |f><i|
    between the quiescent eigenstates (generate_generators.py:459-556)."""
    energies, states = np.linalg.eigh(quiescent)
    temperature = atom.get("T", P.standards.lab.ntp.temperature)
    if temperature > 0:
        b = np.exp(-energies/(math.tau*P.fundamental.boltzmann_gyro*temperature))
    else:
        b = (energies == energies.min()).astype(float)
    out = {}
    for i in range(len(b)):
        for f in range(len(b)):
            den = b[i] + b[f]
            if den == 0:
                continue
            c = math.sqrt(b[f]/(den*T1))
            out[f"L{prefix}1{f} {i}"] = c*np.outer(states[:, f], np.conj(states[:, i]))
    return out


class _Atom:
    """Operators of one atom (electron and/or nucleus) on its block space."""

    def __init__(self, desc):
        self.desc = desc
        self.ops = {}        # label -> matrix (Hamiltonian-like and projectors)
        self.jumps = {}      # label -> matrix (dissipators)
        self.tensors = {}


def _build_spin(atom, kind, P):
    """Operators of one spin of an atom on its own space; returns
    (spin, ops, jumps, projector ops)."""
    d = atom.desc
    ops, jumps, proj_ops = {}, {}, {}
    if kind == "S":
        spin = d.get("S", 0)
        vec, proj = spin_matrices(spin)
        for k, p in proj.items():
            proj_ops["S" + k] = p
        if spin > 0:
            for a, o in zip("xyz", vec):
                ops["S" + a] = o
        zfs = None
        if spin > 0.5:
            D = _zfs_tensor(d.get("D", 0), d.get("E", 0))
            zfs = _quad(D, vec, vec)
            ops["HD"] = zfs
        if spin > 0:
            g = _axial(2, "g", d, "g")
            if "Rb_gets_a" in d:
                g = d["Rb_gets_a"] @ g
            gyro = g*math.tau*P.fundamental.bohr_gyro
            atom.tensors["gyroS"] = gyro
            gen = _lin(gyro, vec)
            for a, o in zip("xyz", gen):
                ops["GS" + a] = o
            jumps.update(_relaxation("S", spin, d, gen, zfs, vec, P))
        return spin, ops, jumps, proj_ops
    spin = d.get("I", 0)
    if spin == 0:
        return 0, ops, jumps, proj_ops
    vec, _ = spin_matrices(spin)
    for a, o in zip("xyz", vec):
        ops["I" + a] = o
    zfs = None
    Pt = _zfs_tensor(d.get("P", 0), d.get("Pt", 0)) if spin > 0.5 else np.zeros((3, 3))
    if np.sum(np.abs(Pt)) > 0:
        zfs = _quad(Pt, vec, vec)
        ops["HP"] = zfs
    g = _axial(2, "gN", d, "gN")
    if "Rb_gets_a" in d:
        g = d["Rb_gets_a"] @ g
    atom.tensors["gyroI"] = -g*math.tau*P.fundamental.nuclear_gyro
    # the quiescent/dephasing generator of the nucleus uses the bare g
    # tensor (generate_generators.py:403-404)
    gen = _lin(g, vec)
    for a, o in zip("xyz", gen):
        ops["GI" + a] = o
    jumps.update(_relaxation("I", spin, d, gen, zfs, vec, P))
    return spin, ops, jumps, proj_ops


def _relaxation(prefix, spin, d, gen, zfs, vec, P):
    jumps = {}
    quiescent_b = None
    if "B0" in d:
        B0 = d["B0"]
        quiescent_b = B0[0]*gen[0] + B0[1]*gen[1] + B0[2]*gen[2]
        if f"T{prefix}2" in d:
            T2 = d[f"T{prefix}2"]
            # the reference tests the element sum of the (re, im) array
            s = np.sum(quiescent_b.real) + np.sum(quiescent_b.imag)
            op = quiescent_b if s > 0 else gen[2]
            l2 = np.max(np.linalg.eigvalsh(op))
            jumps[f"L{prefix}2"] = (spin/(l2*math.sqrt(T2)))*op
    if f"T{prefix}1" in d:
        base = zfs if zfs is not None else np.zeros_like(vec[0])
        q = base.copy() if quiescent_b is None else quiescent_b + base
        jumps.update(_thermal_jumps(prefix, q, d, d[f"T{prefix}1"], P))
    return jumps


# ---------------------------------------------------------------------------
# blocks
# ---------------------------------------------------------------------------

def _add_factor(block_atoms, current, new_ops, new_jumps, new_proj, dim_prev):
    """Join a spin of dimension dim_new to the block (it becomes the fastest
    index); expand every atom's operators accordingly."""
    dims = [m.shape[0] for m in (list(new_ops.values()) + list(new_proj.values()) +
                                 list(new_jumps.values()))]
    dim_new = dims[0] if dims else 1
    I_prev = np.eye(dim_prev, dtype=complex)
    I_new = np.eye(dim_new, dtype=complex)
    if dim_prev > 0:
        for atom in block_atoms:
            for k in list(atom.ops):
                atom.ops[k] = np.kron(atom.ops[k], I_new)
            expanded = {}
            for k, L in atom.jumps.items():
                idx = 0
                for i in range(dim_new):
                    e = np.zeros((dim_new, dim_new), complex)
                    e[i, i] = 1
                    piece = np.kron(L, e)
                    if not np.isclose(np.sum(np.abs(piece)**2), 0):
                        expanded[f"{k} {idx}"] = piece
                    idx += 1
            atom.jumps = expanded
        for k, o in list(new_ops.items()) + list(new_proj.items()):
            current.ops[k] = np.kron(I_prev, o)
        for k, L in new_jumps.items():
            idx = 0
            for o in range(dim_prev):
                e = np.zeros((dim_prev, dim_prev), complex)
                e[o, o] = 1
                piece = np.kron(e, L)
                if not np.isclose(np.sum(np.abs(piece)**2), 0):
                    current.jumps[f"{k} {idx}"] = piece
                idx += 1
        return dim_prev*dim_new
    current.ops.update(new_ops)
    current.ops.update(new_proj)
    current.jumps.update(new_jumps)
    return dim_new


def _build_block(block, interactions, P):
    atoms = [_Atom(copy.deepcopy(d)) for d in block]
    dim = 0
    for atom in atoms:
        s_spin, s_ops, s_jumps, s_proj = _build_spin(atom, "S", P)
        dim = _add_factor(atoms, atom, s_ops, s_jumps, s_proj, dim)
        i_spin, i_ops, i_jumps, i_proj = _build_spin(atom, "I", P)
        if i_spin > 0:
            dim = _add_factor(atoms, atom, i_ops, i_jumps, i_proj, dim)
        atom.s_spin, atom.i_spin = s_spin, i_spin
        _atom_totals(atom)
    couplings = []
    for (ia, ib), jd in interactions.items():
        J = _axial(2, "J", jd, "J")
        la = "S" if "Sx" in atoms[ia].ops else "I"
        lb = "S" if "Sx" in atoms[ib].ops else "I"
        va = tuple(atoms[ia].ops[la + c] for c in "xyz")
        vb = tuple(atoms[ib].ops[lb + c] for c in "xyz")
        couplings.append(_quad(J, va, vb))
    return atoms, dim, couplings


def _atom_totals(atom):
    """Hyperfine, total field generator G, zero-field part Z and quiescent
    H0 of an atom (generate_generators.py:559-681)."""
    o, d = atom.ops, atom.desc
    zero_field = [k for k in ("HD", "HP") if k in o]
    if atom.s_spin > 0 and atom.i_spin > 0:
        A = _axial(2, "A", d, "A")
        o["HA"] = _quad(A, tuple(o["S" + c] for c in "xyz"), tuple(o["I" + c] for c in "xyz"))
        zero_field.append("HA")
    gen = None
    if atom.s_spin > 0:
        gen = _lin(atom.tensors["gyroS"], tuple(o["S" + c] for c in "xyz"))
    if atom.i_spin > 0:
        gi = _lin(atom.tensors["gyroI"], tuple(o["I" + c] for c in "xyz"))
        gen = gi if gen is None else tuple(a + b for a, b in zip(gen, gi))
    if gen is not None:
        for c, g in zip("xyz", gen):
            o["G" + c] = g
    Z = None
    for k in zero_field:
        Z = o[k].copy() if Z is None else Z + o[k]
    if Z is not None:
        o["Z"] = Z
    H0 = None if Z is None else Z.copy()
    if "B0" in d and gen is not None:
        B0 = d["B0"]
        hb = B0[0]*gen[0] + B0[1]*gen[1] + B0[2]*gen[2]
        H0 = hb if H0 is None else H0 + hb
    if H0 is not None:
        o["H0"] = H0


def _traceless(M):
    n = M.shape[0]
    return M - (np.trace(M.real)/n)*np.eye(n)


# ---------------------------------------------------------------------------
# superoperators
# ---------------------------------------------------------------------------

def valid_indices_from_mask(allowed):
    """Diagonal entries first, then upper pairs (y < x) as (re, im)."""
    n = allowed.shape[0]
    rows = [[y, y, 0] for y in range(n) if allowed[y, y]]
    for y in range(n - 1):
        for x in range(y + 1, n):
            if allowed[y, x]:
                rows.append([y, x, 0])
                rows.append([y, x, 1])
    return np.array(rows, dtype=np.int32)


def _basis(n, valid_indices, use_hermitian):
    """Basis matrices B_i (N, n, n) and output selectors (y, x, c)."""
    if use_hermitian:
        y, x, c = valid_indices[:, 0], valid_indices[:, 1], valid_indices[:, 2]
    else:
        i = np.arange(2*n*n)
        c, x, y = i % 2, (i//2) % n, (i//2)//n
    N = len(y)
    B = np.zeros((N, n, n), complex)
    idx = np.arange(N)
    B[idx, y, x] += np.where(c == 1, 1j, 1.0)
    if use_hermitian:
        off = y != x
        B[idx[off], x[off], y[off]] += np.where(c[off] == 1, -1j, 1.0)
    return B, (y, x, c)


def _project(out, sel):
    y, x, c = sel
    vals = out[:, y, x]                    # (in, out)
    return np.where(c[None, :] == 1, vals.imag, vals.real).T.copy()


def von_neumann(H, basis, sel):
    B = basis
    out = -1j*(H[None] @ B - B @ H[None])
    return _project(out, sel)


def dissipator(L, basis, sel):
    B = basis
    Ld = L.conj().T
    LdL = Ld @ L
    out = L[None] @ B @ Ld[None] - 0.5*(LdL[None] @ B + B @ LdL[None])
    return _project(out, sel)


# ---------------------------------------------------------------------------
# inter-block couplings (NV)
# ---------------------------------------------------------------------------

def _states_of(projector):
    return np.where(np.abs(projector).sum(axis=0) > 0)[0]


def _incoherent(initial, final, dim):
    """Jump operators from the states of `initial` to those of `final`
    (pairwise when the counts match, else one all-to-all operator)."""
    si, sf = _states_of(initial), _states_of(final)
    if len(si) == len(sf):
        out = []
        for i, f in zip(si, sf):
            L = np.zeros((dim, dim), complex)
            L[f, i] = 1
            out.append(L)
        return out
    vi = np.abs(initial).sum(axis=0)
    vf = np.abs(final).sum(axis=0)
    return [np.outer(vf, vi).astype(complex)]


def _coherent(initial, final, dim):
    """Hermitian couplings between the states of `initial` and those of
    `final` (reference _couple_coherent, generate_generators.py:2026-2058):
    pairwise when the counts match, else one operator coupling every
    initial state to every final state.  The reference builds the second
    form with a bitwise or on float arrays, which raises a TypeError, so
    that branch follows its evident intent and no fixture pins it."""
    si, sf = _states_of(initial), _states_of(final)
    if len(si) == len(sf):
        out = []
        for i, f in zip(si, sf):
            H = np.zeros((dim, dim), complex)
            H[f, i] = 1
            H[i, f] = 1
            out.append(H)
        return out
    vi = (np.abs(initial).sum(axis=0) > 0).astype(float)
    vf = (np.abs(final).sum(axis=0) > 0).astype(float)
    return [np.maximum(np.outer(vf, vi), np.outer(vi, vf)).astype(complex)]


def _coherent_couplings(a, b, inter, dim, v_index):
    """Coherent (Hamiltonian) couplings of one group interaction between
    m_S states of two blocks (reference generate_generators.py:1503-1525 and
    _couple_coherent_blocks :1961-1991): each entry of inter["coh"] couples
    state `ini` of atom a with state `fin` of atom b at Rabi frequency `amp`
    (rad/s); with "con" true it is controllable (label Vr, scaled by the
    fourth coefficient, into Gr), else constant (Vc, into L0).  Entries
    missing one of ini, fin, amp are skipped.  Returns ({label: operator},
    next v_index); v_index counts couplings over all group interactions.
    (The reference loses its count after an interaction between equal
    spins that has no "rel" rate, and raises at the next coherent coupling;
    the count here simply continues.)"""
    out = {}
    sa, sb = a.desc.get("S"), b.desc.get("S")
    if sa is None or sb is None:
        return out, v_index
    for coh in inter.get("coh", []):
        if not all(k in coh for k in ("ini", "fin", "amp")):
            continue
        label = "Vr" if coh.get("con") else "Vc"
        Pi = a.ops["S" + _proj_key(sa, coh["ini"])]
        Pf = b.ops["S" + _proj_key(sb, coh["fin"])]
        for i, H in enumerate(_coherent(Pi, Pf, dim)):
            out[f"{label} {v_index} {i}"] = H*coh["amp"]
        v_index += 1
    return out, v_index


def _bell(qubit_b, qubit_c, singlet, rates, to_singlet):
    """Jumps between a singlet and the Bell states of two spin-1/2 atoms b and
    c of one block (reference _couple_bell_excited / _couple_bell_ground,
    generate_generators.py:1796-1960): aligned (phi: ++, --) and
    anti-aligned (psi: +-, -+) products of the atoms' projectors.  rates:
    (psi rate, phi rate), None to skip; to_singlet: the jumps run from the
    Bell states to the singlet (ground), else from the singlet (excited)."""
    pb, mb = qubit_b.ops["S" + _proj_key(0.5, 0.5)], qubit_b.ops["S" + _proj_key(0.5, -0.5)]
    pc, mc = qubit_c.ops["S" + _proj_key(0.5, 0.5)], qubit_c.ops["S" + _proj_key(0.5, -0.5)]
    s = singlet.ops["S" + _proj_key(0, 0)]
    states = {"psi+": pb*mc, "psi-": mb*pc, "phi+": pb*pc, "phi-": mb*mc}
    dim = s.shape[0]
    out = {}
    for kind, rate in zip(("psi", "phi"), rates):
        if rate is None:
            continue
        for sign in "+-":
            proj = states[kind + sign]
            jumps = _incoherent(proj, s, dim) if to_singlet else _incoherent(s, proj, dim)
            for i, L in enumerate(jumps):
                label = f"Lbell {kind}{sign} g {i}" if to_singlet else f"Lbell e {kind}{sign} {i}"
                out[label] = L*math.sqrt(rate)
    return out


def _block_coupling(a, b, inter, dim, label_prefix, next_a=None, next_b=None):
    """Jumps of one group interaction; returns {label: operator}.  next_a,
    next_b: the atoms after a and b in their blocks (the second qubit of a
    Bell pair), or None."""
    out = {}
    sa, sb = a.desc.get("S"), b.desc.get("S")
    if sa is None or sb is None:
        return out

    def P(atom, spin, m):
        return atom.ops["S" + _proj_key(spin, m)]

    if sa == sb:
        if "rel" not in inter:
            return out
        rel, reln = inter["rel"], inter.get("rel_n")
        for m in np.arange(-sa, sa + 0.1):
            n = _num(sa, m)
            for i, L in enumerate(_incoherent(P(a, sa, m), P(b, sb, m), dim)):
                out[f"Lrc{n} {n} {i}"] = L*math.sqrt(rel)
            for i, L in enumerate(_incoherent(P(b, sb, m), P(a, sa, m), dim)):
                out[f"Llc{n} {n} {i}"] = L*math.sqrt(rel)
            if reln is None:
                continue
            for me in np.arange(-sa, sa + 0.1):
                if not np.isclose(abs(m - me), 1):
                    continue
                ne = _num(sa, me)
                for i, L in enumerate(_incoherent(P(a, sa, m), P(b, sb, me), dim)):
                    r = reln/2 if np.isclose(abs(m), sa) else reln
                    out[f"Lrn{ne} {n} {i}"] = L*math.sqrt(r)
                for i, L in enumerate(_incoherent(P(b, sb, me), P(a, sa, m), dim)):
                    r = reln/2 if np.isclose(abs(me), sa) else reln
                    out[f"Lln{n} {ne} {i}"] = L*math.sqrt(r)
    elif sa == 1 and sb == 0:
        r0, r1 = inter.get("s_gets_0"), inter.get("s_gets_1")
        for m in np.arange(-1, 1.1):
            n = _num(1, m)
            rate = r0 if np.isclose(m, 0) else r1
            if rate is None:
                continue
            for i, L in enumerate(_incoherent(P(a, 1, m), P(b, 0, 0), dim)):
                out[f"Lisc s {n} {i}"] = L*np.sqrt(rate)
    elif sa == 0 and sb == 1:
        r0, r1 = inter.get("0_gets_s"), inter.get("1_gets_s")
        for m in np.arange(-1, 1.1):
            n = _num(1, m)
            rate = r0 if np.isclose(m, 0) else r1
            if rate is None:
                continue
            for i, L in enumerate(_incoherent(P(a, 0, 0), P(b, 1, m), dim)):
                out[f"Lisc{n} s {i}"] = L*np.sqrt(rate)
    elif sa == 0 and sb == 0.5:
        # singlet a decays to the Bell states of atom b and the next atom
        rates = (inter.get("psi_gets_e"), inter.get("phi_gets_e"))
        if rates != (None, None):
            if next_b is None:
                raise ValueError("a Bell coupling needs the atom after the qubit in its block")
            out.update(_bell(b, next_b, a, rates, to_singlet=False))
    elif sa == 0.5 and sb == 0:
        # the Bell states of atom a and the next atom decay to singlet b
        rates = (inter.get("g_gets_psi"), inter.get("g_gets_phi"))
        if rates != (None, None):
            if next_a is None:
                raise ValueError("a Bell coupling needs the atom after the qubit in its block")
            out.update(_bell(a, next_a, b, rates, to_singlet=True))
    return out


# ---------------------------------------------------------------------------
# entry point
# ---------------------------------------------------------------------------

def generate_atoms(description, atom_interactions, block_interactions, use_unitary=False,
                   use_hermitian=True, use_incoherent=True, verbose=False, params=None):
    """Generators of a spin system (reference generate_generators.py:19-166).

    Returns (operators, valid_indices): ``operators["generators"]`` holds
    the real (N, N) superoperators L0, Gx, Gy, Gz, Gr; ``valid_indices`` is
    the (N, 3) vectorisation map (rows y, x, c).
    """
    P = params or default_params
    if not use_hermitian:
        use_incoherent = False
    blocks = []
    for b, (block, inter) in enumerate(zip(description, atom_interactions)):
        atoms, dim, couplings = _build_block(block, inter, P)
        for atom in atoms:
            for k in list(atom.ops):
                if "|" not in k:
                    atom.ops[k] = _traceless(atom.ops[k])
        blocks.append((atoms, max(dim, 1), couplings))
    # blocks joined by coherent couplings, closed transitively (generate_
    # generators.py:76-91): their mutual coherences are allowed entries
    nb = len(blocks)
    joined = np.eye(nb, dtype=bool)
    for ((ba, _), (bb, _)), inter in block_interactions.items():
        if "coh" in inter:
            joined[ba, bb] = joined[bb, ba] = True
    while True:
        grown = joined.copy()
        for c in range(nb):
            grown |= np.outer(joined[c], joined[c])
        if (grown == joined).all():
            break
        joined = grown
    sizes = [d for _, d, _ in blocks]
    n = sum(sizes)
    offsets = np.cumsum([0] + sizes)

    def embed(M, b):
        out = np.zeros((n, n), complex)
        o = offsets[b]
        out[o:o + M.shape[0], o:o + M.shape[1]] = M
        return out

    coherent = {}
    jumps = {}
    for b, (atoms, dim, couplings) in enumerate(blocks):
        block_sum = {}
        for a_idx, atom in enumerate(atoms):
            for k in ("Gx", "Gy", "Gz", "Z", "H0"):
                if k in atom.ops:
                    block_sum[k] = block_sum.get(k, 0) + atom.ops[k]
            for k, L in atom.jumps.items():
                jumps[f"[{b}, {a_idx}] {k}"] = embed(L, b)
            for k in list(atom.ops):
                atom.ops[k] = embed(atom.ops[k], b)
        for Hj in couplings:
            for k in ("Z", "H0"):
                block_sum[k] = block_sum.get(k, 0) + Hj
        for k, M in block_sum.items():
            coherent[k] = coherent.get(k, 0) + embed(M, b)
    couplings_h = {}
    v_index = 0
    for ((ba, aa), (bb, ab)), inter in block_interactions.items():
        atoms_a, atoms_b = blocks[ba][0], blocks[bb][0]
        atom_a, atom_b = atoms_a[aa], atoms_b[ab]
        hs, v_index = _coherent_couplings(atom_a, atom_b, inter, n, v_index)
        for k, H in hs.items():
            couplings_h[f"[{ba}, {aa}, {bb}, {ab}] {k}"] = H
        nxt_a = atoms_a[aa + 1] if aa + 1 < len(atoms_a) else None
        nxt_b = atoms_b[ab + 1] if ab + 1 < len(atoms_b) else None
        for k, L in _block_coupling(atom_a, atom_b, inter, n, "", nxt_a, nxt_b).items():
            jumps[f"[{ba}, {aa}, {bb}, {ab}] {k}"] = L

    allowed = np.zeros((n, n), int)
    for b in range(nb):
        o = offsets[b]
        allowed[o:o + sizes[b], o:o + sizes[b]] = 1
    for b1 in range(nb):
        for b2 in range(nb):
            if joined[b1, b2]:
                allowed[offsets[b1]:offsets[b1 + 1], offsets[b2]:offsets[b2 + 1]] = 1
    if not use_incoherent:
        allowed[:] = 1
    valid = valid_indices_from_mask(allowed)
    if use_unitary and not jumps and couplings_h:
        raise NotImplementedError("unitary mode with coherent block couplings")
    if use_unitary and not jumps:
        # closed system: operator generators and the basis change matrices
        # (generate_generators.py:120-139); no superoperators
        unitary = {k: complex_to_real(coherent.get(k, np.zeros((n, n), complex)))
                   for k in ("H0", "Gx", "Gy", "Gz", "Z")}
        unitary["Gr"] = np.zeros((2*n, 2*n))
        elim, dup = elimination_matrices(n, valid, use_hermitian)
        return {"unitary": unitary, "elimination": {"elimination": elim, "duplication": dup},
                "coherent": coherent, "jump": jumps, "allowed": allowed}, valid
    basis, sel = _basis(n, valid, use_hermitian)

    supers = {}
    for k, L in jumps.items():
        supers[k] = dissipator(L, basis, sel)
    for k, H in coherent.items():
        supers[k] = von_neumann(H, basis, sel)
    for k, H in couplings_h.items():
        supers[k] = von_neumann(H, basis, sel)
    generators = _group(supers)
    return {"generators": generators, "super_all": supers, "coherent": coherent,
            "coherent_coupling": couplings_h, "jump": jumps, "allowed": allowed}, valid


def _group(supers):
    """L0 = H0 + D + Vc; Gr = controllable jumps (generate_generators.py:
    2226-2314)."""
    stage1 = {}
    for label, S in supers.items():
        if "]" not in label:
            continue
        atom, op = label.split("] ", 1)
        for pre in JUMP_PREFIXES:
            if len(op) > len(pre) and op.startswith(pre):
                key = (atom, pre)
                stage1[key] = stage1.get(key, 0) + S
    per_atom = {}
    exact = [(label.split("] ", 1)[0], label.split("] ", 1)[1], S)
             for label, S in supers.items() if "]" in label]
    exact += [(a, p, S) for (a, p), S in stage1.items()]
    for atom, op, S in exact:
        for group, members in GROUPS.items():
            if op in members:
                key = (atom, group)
                per_atom[key] = per_atom.get(key, 0) + S
    totals = {}
    for (atom, group), S in per_atom.items():
        totals[group] = totals.get(group, 0) + S
    N = next(iter(supers.values())).shape[0]
    zero = np.zeros((N, N))
    L0 = zero.copy()
    for k in ("H0", "D", "Vc"):
        if k == "H0" and "H0" in supers:
            L0 = L0 + supers["H0"]
        elif k in totals:
            L0 = L0 + totals[k]
    out = {"L0": L0}
    for k in ("Gx", "Gy", "Gz"):
        out[k] = supers.get(k, zero.copy())
    out["Gr"] = totals.get("Gr", zero.copy())
    return out


# ---------------------------------------------------------------------------
# unitary representation
# ---------------------------------------------------------------------------

def complex_to_real(H):
    """Real 2n x 2n form of i*H acting on interleaved (re, im) vectors: entry
    (i, j) of the complex matrix iH sits at [2i][2j] (real part) and
    [2i+1][2j] (imaginary part), with [2i][2j+1] = -imag and [2i+1][2j+1] =
    real.  This is the reference's operator generator
    (generate_generators.py:2725-2746), the real form of +iH."""
    Z = 1j*np.asarray(H, dtype=complex)
    n = Z.shape[0]
    out = np.empty((2*n, 2*n))
    out[::2, ::2] = Z.real
    out[1::2, ::2] = Z.imag
    out[::2, 1::2] = -Z.imag
    out[1::2, 1::2] = Z.real
    return out


def elimination_matrices(n, valid_indices, use_hermitian):
    """Elimination (N_h x 2n^2) and duplication (2n^2 x N_h) matrices between
    the Hermitian basis of the vectorisation map and the full basis of all
    (y, x, re/im) entries listed column-major, each entry the overlap of two
    basis matrices over the squared norm of the first
    (generate_generators.py:2797-2840)."""
    full = np.zeros((2*n*n, n, n, 2))
    k = 0
    for x in range(n):
        for y in range(n):
            for c in range(2):
                full[k, y, x, c] = 1.0
                k += 1
    if use_hermitian:
        herm = np.zeros((len(valid_indices), n, n, 2))
        for i, (y, x, c) in enumerate(valid_indices):
            herm[i, y, x, c] = 1.0
            if y != x:
                herm[i, x, y, c] = -1.0 if c else 1.0
    else:
        herm = full.copy()
    fh = herm.reshape(len(herm), -1)
    ff = full.reshape(len(full), -1)
    elim = (fh @ ff.T)/np.sum(fh**2, axis=1)[:, None]
    dup = (ff @ fh.T)/np.sum(ff**2, axis=1)[:, None]
    return elim, dup


# ---------------------------------------------------------------------------
# equivalence classes (common kernel of the generators)
# ---------------------------------------------------------------------------

def _gram_schmidt(vectors, avoid=(), tolerance=1e-14):
    out = []
    for v in vectors:
        v = np.array(v, dtype=np.float64)
        for d in avoid:
            v -= np.dot(d, v)*d
        for d in out:
            v -= np.dot(d, v)*d
        nrm = np.linalg.norm(v)
        if nrm < tolerance:
            continue
        out.append(v/nrm)
    return out


def find_kernel(generators, rtol=1e-9):
    """(full basis, image basis, generators on the image) for the common
    kernel of the generators (reference generate_generators.py:2691-2719).

    The reference takes each generator's kernel from eigenvectors with
    |lambda| <= max|lambda|/1e9, makes the bases real and intersects them
    (Zassenhaus).  The common kernel is the null space of the stacked
    generators, found here by SVD of the generators scaled to unit norm with
    the same relative threshold.  The image basis is then Gram-Schmidt of the
    identity's columns against the kernel, as the reference's
    _find_orthogonal does (:2667-2688), and the generators are restricted to
    it: image^T G image.  Without a common kernel all three are the
    identity / the generators themselves."""
    gens = [np.asarray(g, dtype=np.float64) for g in generators]
    N = gens[0].shape[0]
    rows = [g/np.linalg.norm(g, 2) for g in gens if np.any(g != 0)]
    if not rows:
        kernel = np.eye(N)
    else:
        _, sv, vt = np.linalg.svd(np.vstack(rows))
        sv = np.concatenate([sv, np.zeros(N - sv.size)])
        kernel = vt[sv <= rtol*sv.max()]
    if len(kernel) == 0:
        return np.eye(N), np.eye(N), gens
    # orient each kernel vector with a positive leading entry, as the
    # reference's row-echelon basis comes out
    kernel = np.array([k if k[np.argmax(np.abs(k) > 1e-12)] > 0 else -k for k in kernel])
    korth = _gram_schmidt(kernel)
    image = _gram_schmidt(np.eye(N), korth)
    image_a = np.array(image).T
    full = np.array(image + korth).T
    return full, image_a, [image_a.T @ g @ image_a for g in gens]
