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
                           use_incoherent=c["use_incoherent"])
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


def test_unsupported_raise():
    with pytest.raises(NotImplementedError):
        generate_atoms([[{"S": 1}]], [{}], {}, use_unitary=True)


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
