"""The CPU oracle against the reference's own outputs (no GPU).

The fixtures in tests/golden were produced by the reference itself
(tests/golden/make_golden.py); the golden CSV prefixes are the reference's
regression vectors (test/reference/*.csv in the reference)."""
import numpy as np
import pytest

from conftest import load_case, quadrature
from oracle import oracle

CASES = ["qubit_couple", "qubit_couple_res_e2", "qubit_couple_res_e2_cpu",
         "qubit_couple_res_e5", "qubit_couple_res_e3_e6", "qubit_t1_0K",
         "qubit_t1_mK", "qutrit_couple", "qutrit_couple_unital",
         "qubit_hyperfine", "qubit_couple_rot_e5",
         "qubit_couple_rot_e1_nores", "spin1_c1", "nv7_n49", "nv7_n19",
         "qubit_couple_nh", "qubit_couple_rot_nh", "qubit_t1_0K_rot",
         "qubit_t1_mK_rot_e2", "coherent_chain", "hbn_bell"]


def vmap(c):
    """The case's vectorisation map; none in the complex (non-Hermitian)
    basis, whose entries are (y, x, re/im) in row-major order."""
    return c["vectorisation_map"] if bool(c.get("meta_herm", True)) else None


def run(c, mode="reference", T=None, K=None, degree=14, dt=None):
    K = K or int(c["meta_K"])
    W, nodes = quadrature(K)
    rot = None
    if bool(c["meta_rot"]):
        rot = dict(generators_rotating=c["generators_rotating"],
                   vectors_real=c["vectors_real"],
                   inv_vectors_real=c["inv_vectors_real"],
                   doubles=c["doubles"], singles=c["singles"])
    if T is None:
        t0, tf, dt = c["times"]
    else:
        t0, tf = 0.0, T*dt + dt*1e-4
    return oracle.simulate(
        c["generators"], c["rho0"], t0, tf, dt, c["program"], K=K, W=W,
        nodes=nodes, F=int(c["meta_F"]), R=int(c["meta_R"]),
        residual=bool(c["meta_res"]),
        vectorisation_map=vmap(c), rotating=rot, mode=mode,
        degree=degree)


@pytest.mark.parametrize("name", CASES)
def test_reference_mode_matches_reference(name):
    c = load_case(name)
    t, d = run(c)
    assert d.shape == c["density"].shape
    t0, tf, dt = c["times"]
    assert np.array_equal(t, t0 + dt*(np.arange(d.shape[0]) + 1))
    # bit-exact on the machine that made the fixtures; libm cos may differ
    # by an ulp elsewhere
    assert np.abs(d - c["density"]).max() <= 1e-14
    if "density_K6" in c:
        _, d6 = run(c, K=6)
        assert np.abs(d6 - c["density_K6"]).max() <= 1e-14


@pytest.mark.parametrize("name", [n for n in CASES if "nores" not in n
                                  and n != "qubit_couple"])
def test_vector_mode_matches_reference_mode(name):
    c = load_case(name)
    _, d = run(c, mode="vector")
    assert np.abs(d - c["density"]).max() <= 1e-13


def _flat29(d):
    e = np.empty(d.shape + (2,))
    e[..., 0], e[..., 1] = d.real, d.imag
    return e.flatten()[::29]


@pytest.mark.parametrize("name,nvals,tol", [
    ("qubit_couple", 400, 1e-10), ("qubit_t1_0K", 400, 1e-14),
    ("qubit_t1_mK", 400, 1e-14), ("qutrit_couple", 400, 1e-14),
    ("qutrit_couple_unital", 400, 1e-14), ("qubit_hyperfine", 200, 1e-14),
    ("qutrit_hyperfine", 60, 1e-14), ("qubit_couple_rot_nh", 400, 1e-6)])
def test_reference_golden_csv_prefix(name, nvals, tol):
    """The reference's golden regression vectors (generated on its GPU
    path, 1 ns output grid, F = 100).  The complex-basis rotating case is
    the reference's qubit-couple-res-rot-nh.py, which checks its run
    against qubit-couple.csv -- made in plain (non-residual) lab-frame
    arithmetic -- with a root-sum-square bar of 1e-5: the two drift apart
    as about t^2 (3e-9 at 100 ns, 3.4e-7 after the 1.45 us this prefix
    spans).  Its own output is pinned to 1e-14 by the fixture above."""
    c = load_case(name)
    n = c["rho0"].shape[0]
    T = int(np.ceil(nvals*29/(2*n*n))) + 1
    _, d = run(c, T=T, dt=1e-9)
    f = _flat29(d)[:nvals]
    assert np.abs(f - c["csv_prefix"][:nvals]).max() <= tol


def test_sample_count_truncates():
    # generate_simulator.py:1519 -- int((tf - t0)/dt): 100 ns / 1 ns -> 99
    assert oracle.number_of_samples(0, 100e-9, 1e-9) == 99


def test_flatten_roundtrip():
    c = load_case("nv7_n49")
    vm = c["vectorisation_map"]
    rng = np.random.default_rng(1)
    a = rng.normal(size=(7, 7)) + 1j*rng.normal(size=(7, 7))
    h = a + a.conj().T
    f = oracle.flatten(h, vm, vm.shape[0])
    assert np.allclose(oracle.unflatten(f, vm, 7), h, atol=0, rtol=0)
