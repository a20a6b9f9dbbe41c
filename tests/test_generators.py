"""The generator builder against the reference's own generators (no GPU)."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, load_case

sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402  (case definitions only; the reference is not imported)

from superspinsim_gb300 import models  # noqa: E402
from superspinsim_gb300.generators import generate_atoms  # noqa: E402

LABELS = ["L0", "Gx", "Gy", "Gz", "Gr"]


@pytest.mark.parametrize("c", make_golden.cases(), ids=lambda c: c["name"])
def test_generators_match_reference(c):
    z = load_case(c["name"])
    g, vm = generate_atoms(c["spins"], c["spin_interactions"], c["group_interactions"],
                           use_incoherent=c["use_incoherent"],
                           use_hermitian=c.get("herm", True))
    gens = np.array([g["generators"][k] for k in LABELS])
    assert np.array_equal(vm, z["vectorisation_map"])
    ref = z["generators"]
    assert gens.shape == ref.shape
    for i in range(5):
        scale = max(1.0, np.abs(ref[i]).max())
        assert np.abs(gens[i] - ref[i]).max() <= 1e-15*scale


@pytest.mark.parametrize("name,incoherent", [("nv7_n49", False), ("nv7_n19", True)])
def test_nv7_model_matches_reference(name, incoherent):
    z = load_case(name)
    spins, inter, groups = models.nv_7(np.array([0, 0, 5e-3]), params=models.odmr_params())
    g, vm = generate_atoms(spins, inter, groups, use_incoherent=incoherent)
    gens = np.array([g["generators"][k] for k in LABELS])
    assert np.array_equal(vm, z["vectorisation_map"])
    for i in range(5):
        scale = max(1.0, np.abs(z["generators"][i]).max())
        assert np.abs(gens[i] - z["generators"][i]).max() <= 1e-15*scale


def test_lindbladian_properties():
    """Trace preservation: the population-sum functional is conserved by
    every generator (columns of the diagonal rows sum to zero)."""
    spins, inter, groups = models.nv_7(np.array([0, 0, 5e-3]))
    g, vm = generate_atoms(spins, inter, groups, use_incoherent=False)
    diag = np.array([1.0 if y == x and c == 0 else 0.0 for y, x, c in vm])
    for k in LABELS:
        assert np.abs(diag @ g["generators"][k]).max() <= 1e-6*max(1, np.abs(g["generators"][k]).max())*1e-6


@pytest.mark.parametrize("name", ["qubit", "qutrit", "qubit_hf"])
def test_unitary_generators_and_elimination_match_reference(name):
    """Operator generators (real form of +iH), elimination/duplication
    matrices and the map, against the reference's own output."""
    import make_golden as mg
    spins = {"qubit": mg.QUBIT, "qutrit": mg.QUTRIT, "qubit_hf": mg.QUBIT_HF}[name]
    z = np.load(os.path.join(GOLDEN, f"modes_{name}.npz"))
    ops, vm = generate_atoms(spins, [{}], {}, use_unitary=True)
    for k in ("H0", "Gx", "Gy", "Gz", "Gr"):
        assert np.array_equal(ops["unitary"][k], z["unitary_" + k]), k
    assert np.array_equal(ops["elimination"]["elimination"], z["elimination"])
    assert np.array_equal(ops["elimination"]["duplication"], z["duplication"])
    assert np.array_equal(vm, z["vectorisation_map"])


def test_unitary_falls_back_with_jump_operators():
    ops, _ = generate_atoms([[{"S": 1/2, "g": 2.0, "B0": np.array([0, 0, 1e-3]),
                               "TS2": 1e-6}]], [{}], {}, use_unitary=True)
    assert "unitary" not in ops and "generators" in ops


@pytest.mark.parametrize("name", ["qubit", "qutrit", "qubit_hf"])
def test_find_kernel_matches_reference(name):
    """Image basis and projected generators against the reference's
    find_kernel.  On the hyperfine qubit the reference finds no common
    kernel although the identity direction is annihilated by every
    generator; there the restatement removes it (r = 15), and the
    projection is exact, so both give the same dynamics."""
    from superspinsim_gb300.generators import find_kernel
    z = np.load(os.path.join(GOLDEN, f"modes_{name}.npz"))
    gens = z["generators"]
    full, image, gi = find_kernel(list(gens))
    if name == "qubit_hf":
        assert z["image_projection"].shape[1] == 16 and image.shape[1] == 15
        k = full[:, 15]
        for g in gens:
            assert np.abs(g @ k).max() <= 1e-9*np.abs(g).max()
        return
    assert np.abs(image - z["image_projection"]).max() <= 1e-14
    assert np.abs(full - z["full_projection"]).max() <= 1e-14
    scale = np.abs(gens).max()
    assert np.abs(np.array(gi) - z["generators_image"]).max() <= 1e-14*scale


@pytest.mark.parametrize("name", ["qubit_hyperfine", "qubit_couple_rot_e5", "qutrit_hyperfine"])
def test_make_rotating_matches_reference(name):
    from superspinsim_gb300.rotating import make_rotating
    z = load_case(name)
    g = z["generators"]
    new, V, Vi, d, s = make_rotating(g[0], list(g[1:]))
    # V is a basis: V^-1 V = I
    assert np.abs(Vi @ V - np.eye(V.shape[0])).max() <= 1e-9
    scale = np.abs(g).max()
    # and equals the reference's frame on the machine that made the fixtures
    assert np.abs(V - z["vectors_real"]).max() <= 1e-12
    assert np.abs(np.array(new) - z["generators_rotating"]).max() <= 1e-9*scale


def test_nv21_model_matches_reference():
    """21-level NV with 14N (441 x 441 Liouvillian)."""
    z = load_case("nv21_n441")
    spins, inter, groups = models.nv_21(np.array([0, 0, 0.05]), params=models.nv21_params())
    g, vm = generate_atoms(spins, inter, groups, use_incoherent=False)
    assert np.array_equal(vm, z["vectorisation_map"])
    for i, k in enumerate(LABELS):
        ref = z["generators"][i]
        assert np.abs(g["generators"][k] - ref).max() <= 1e-15*np.abs(ref).max()


def test_coherent_couplings_labels_and_closure():
    """Coherent block couplings: one Hermitian operator per coupled state
    pair, labelled Vc (constant, into L0) or Vr (into Gr) with the running
    coupling index; blocks 0 and 2, joined only through block 1, have their
    coherences allowed by the transitive closure, and an uncoupled fourth
    block does not."""
    spins, inter, groups = make_golden.coherent_chain()
    ops, vm = generate_atoms(spins, inter, groups)
    hs = ops["coherent_coupling"]
    assert sorted(hs) == ["[0, 0, 1, 0] Vc 0 0", "[1, 0, 2, 0] Vr 1 0"]
    for H in hs.values():
        assert np.array_equal(H, H.conj().T) and np.count_nonzero(H) == 2
    allowed = ops["allowed"]
    assert allowed.shape == (7, 7) and allowed.all()
    # an extra uncoupled qubit block: its coherences with the chain stay out
    ops4, vm4 = generate_atoms(spins + [[{"S": 1/2, "g": 2.0, "B0": make_golden.B0}]],
                               inter + [{}], groups)
    a4 = ops4["allowed"]
    assert a4[:7, :7].all() and not a4[:7, 7:].any() and a4[7:, 7:].all()
    # the Vr coupling is the only controllable term: Gr is exactly its
    # von Neumann superoperator
    assert np.abs(ops["generators"]["Gr"]).max() > 0


def test_bell_couplings_labels():
    """hBN-style Bell couplings: the singlet decays to each of the four Bell
    product states of the pair and back, sqrt(rate) scaled jumps."""
    spins, inter, groups = make_golden.hbn_bell()
    ops, _ = generate_atoms(spins, inter, groups)
    labels = sorted(k.split("] ", 1)[1] for k in ops["jump"] if "Lbell" in k)
    want = sorted([f"Lbell e {s} 0" for s in ("psi+", "psi-", "phi+", "phi-")] +
                  [f"Lbell {s} g 0" for s in ("psi+", "psi-", "phi+", "phi-")])
    assert labels == want
    L = ops["jump"]["[1, 0, 0, 0] Lbell e psi+ 0"]
    assert np.isclose(np.abs(L).max(), np.sqrt(2e7))
    L = ops["jump"]["[0, 0, 1, 0] Lbell phi- g 0"]
    assert np.isclose(np.abs(L).max(), np.sqrt(1e6))
    with pytest.raises(ValueError):
        # the pair's second atom is missing
        generate_atoms([[spins[0][0]], spins[1]], [{}, {}], groups)
