"""CUDA path (through the C-ABI) against the oracle on the reference's own
fixtures.  Tolerances: max-abs on the density matrix elements."""
import numpy as np
import pytest

from conftest import load_case, quadrature
from oracle import oracle

pytestmark = pytest.mark.gpu

CASES = ["qubit_couple_res_e2", "qubit_couple_res_e5", "qubit_couple_res_e3_e6",
         "qubit_t1_0K", "qubit_t1_mK", "qutrit_couple", "qutrit_couple_unital",
         "qubit_hyperfine", "qubit_couple_rot_e5", "spin1_c1", "nv7_n49",
         "nv7_n19", "qubit_couple_nh", "qubit_couple_rot_nh", "qubit_t1_0K_rot",
         "qubit_t1_mK_rot_e2", "coherent_chain", "hbn_bell"]
NONRES = ["qubit_couple", "qubit_couple_rot_e1_nores"]


def _sim(c, expm, K=None, T=None, dt=None, F=None):
    from superspinsim_gb300 import generate_simulator
    K = K or int(c["meta_K"])
    rot = bool(c["meta_rot"])
    kw = {}
    if rot:
        kw = dict(use_rotating=True, vectors_real=c["vectors_real"],
                  inv_vectors_real=c["inv_vectors_real"], doubles=c["doubles"],
                  singles=c["singles"])
        gens = c["generators_rotating"]
    else:
        gens = c["generators"]
    herm = bool(c.get("meta_herm", True))
    sim = generate_simulator(
        c["program"], gens, c["vectorisation_map"] if herm else None, use_hermitian=herm,
        use_residual=bool(c["meta_res"]), number_of_quartic_repeats=int(c["meta_R"]),
        number_of_exponentials=K, number_of_fine_divisions=F or int(c["meta_F"]),
        expm=expm, **kw)
    if T is None:
        t0, tf, dt = c["times"]
    else:
        t0, tf = 0.0, T*dt + dt*1e-4
    return sim(c["rho0"], t0, tf, dt)


@pytest.mark.parametrize("expm", ["taylor", "reference"])
@pytest.mark.parametrize("name", CASES)
def test_simulate_matches_reference_fixture(name, expm):
    c = load_case(name)
    t, d = _sim(c, expm)
    t0, tf, dt = c["times"]
    assert np.array_equal(t, t0 + dt*(np.arange(d.shape[0]) + 1))
    assert d.shape == c["density"].shape
    assert np.abs(d - c["density"]).max() <= 1e-12
    if "density_K6" in c:
        _, d6 = _sim(c, expm, K=6)
        assert np.abs(d6 - c["density_K6"]).max() <= 1e-12


@pytest.mark.parametrize("name", NONRES)
def test_non_residual_reference_arithmetic(name):
    """Non-residual mode adds the identity before 2R squarings, which loses
    the small diagonal terms (reference arithmetic); the reference
    algorithm reproduces it, the Taylor one is more accurate."""
    c = load_case(name)
    _, d = _sim(c, "reference")
    assert np.abs(d - c["density"]).max() <= 1e-12
    _, d2 = _sim(c, "taylor")
    assert np.abs(d2 - c["density"]).max() <= 1e-9


@pytest.mark.parametrize("name,T,dt,F", [("spin1_c1", 30, 1e-9, 100),
                                         ("nv7_n49", 3, 1e-9, 200),
                                         ("nv7_n19", 6, 1e-9, 200),
                                         ("qubit_hyperfine", 40, 1e-9, 100),
                                         ("qubit_couple_rot_nh", 40, 1e-9, 100)])
def test_longer_window_against_oracle(name, T, dt, F):
    c = load_case(name)
    K = int(c["meta_K"])
    W, nodes = quadrature(K)
    rot = None
    if bool(c["meta_rot"]):
        rot = dict(generators_rotating=c["generators_rotating"],
                   vectors_real=c["vectors_real"], inv_vectors_real=c["inv_vectors_real"],
                   doubles=c["doubles"], singles=c["singles"])
    _, ref = oracle.simulate(c["generators"], c["rho0"], 0.0, T*dt + dt*1e-4, dt,
                             c["program"], K=K, W=W, nodes=nodes, F=F,
                             residual=bool(c["meta_res"]),
                             vectorisation_map=c["vectorisation_map"]
                             if bool(c.get("meta_herm", True)) else None, rotating=rot,
                             mode="vector", degree=16)
    _, d = _sim(c, "taylor", T=T, dt=dt, F=F)
    assert np.abs(d - ref).max() <= 1e-11


def test_callable_sampler_matches_program():
    """A plain Python sampler (host-sampled table) gives the same result as
    the device-evaluated program."""
    from superspinsim_gb300 import generate_simulator
    from superspinsim_gb300.program import array_value
    c = load_case("qutrit_couple")
    prog = c["program"]

    def sampler(time, row):
        row[0] = 1.0
        for ch in range(4):
            row[ch + 1] = array_value(prog, ch, time)

    kw = dict(use_residual=True, number_of_exponentials=2, number_of_fine_divisions=20)
    s1 = generate_simulator(prog, c["generators"], c["vectorisation_map"], **kw)
    s2 = generate_simulator(sampler, c["generators"], c["vectorisation_map"], **kw)
    _, d1 = s1(c["rho0"], 0.0, 5e-9, 1e-9)
    _, d2 = s2(c["rho0"], 0.0, 5e-9, 1e-9)
    assert np.abs(d1 - d2).max() <= 1e-15


def test_empty_window_and_errors():
    from superspinsim_gb300 import generate_simulator
    c = load_case("qubit_couple_res_e2")
    sim = generate_simulator(c["program"], c["generators"], c["vectorisation_map"])
    t, d = sim(c["rho0"], 0.0, 0.5e-9, 1e-9)
    assert t.shape == (0,) and d.shape == (0, 2, 2)
    with pytest.raises(NotImplementedError):
        generate_simulator(c["program"], c["generators"], use_cuda=False)
    with pytest.raises(TypeError):
        generate_simulator(c["program"], c["generators"], use_cayley=True)


def _case_by_name(name):
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import make_golden
    for c in make_golden.cases():
        if c["name"] == name:
            return c, make_golden
    raise KeyError(name)


@pytest.mark.parametrize("name", ["qubit_couple_res_e2", "qubit_t1_mK", "qutrit_couple",
                                  "qubit_hyperfine", "qubit_couple_rot_e5", "spin1_c1",
                                  "qubit_couple_rot_nh", "coherent_chain", "hbn_bell"])
def test_simspins_front_end_matches_reference(name):
    """The whole front end -- this package's generator builder, rotating
    frame and simulator -- against the reference's simspins output."""
    from superspinsim_gb300.sugar import simspins
    c, mg = _case_by_name(name)
    ref = load_case(name)
    fns = [mg.channel_fn(s) for s in c["ch"]]
    t0, tf, dt = c["t"]
    _, d = simspins(fns, t0, tf, dt, c["spins"], c["spin_interactions"],
                    c["group_interactions"], c["rho0"], number_of_exponentials=c["K"],
                    number_of_fine_divisions=c["F"], number_of_quadratic_repeats=c["R"],
                    use_rotating=c["rot"], use_residual=c["res"],
                    use_incoherent=c["use_incoherent"], use_hermitian=c.get("herm", True))
    assert np.abs(d - ref["density"]).max() <= 1e-12


def test_mesolve_front_end_matches_reference():
    """QuTiP-style front end against the reference's mesolve (static jump
    operators, rotating frame, CF6:5, F = 10)."""
    from superspinsim_gb300.sugar import mesolve
    c, mg = _case_by_name("qubit_couple")   # only for the module handle
    H, c_ops, rho0 = mg.mesolve_case()
    ref = load_case("mesolve_qubit")["density"]
    _, d = mesolve(H, rho0, 0.0, 20e-9, 1e-9, c_ops=c_ops, number_of_exponentials=5,
                   number_of_fine_divisions=10)
    assert np.abs(d - ref).max() <= 1e-12
