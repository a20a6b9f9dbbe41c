"""Batched runs in the generalised rotating frame (row-part kernel with the
e^{L0 h} step and the eigenbasis changes) against the reference's own
rotating-frame output and against the oracle's rotating mode."""
import numpy as np
import pytest

from conftest import load_case, quadrature
from oracle import oracle

pytestmark = pytest.mark.gpu

F_RES = 2.870e9 + 28.025e9*5e-3


def _odmr_programs(freqs, amp, laser):
    progs = np.zeros((len(freqs), 4, 1, 5))
    progs[:, :, :, 0] = np.inf
    progs[:, 0, 0, 2] = amp
    progs[:, 0, 0, 3] = freqs
    progs[:, 3, 0, 1] = laser
    return progs


def _excited_weights(vmap):
    w = np.zeros(vmap.shape[0])
    for i, (y, x, c) in enumerate(vmap):
        if y == x and y in (3, 4, 5) and c == 0:
            w[i] = 1.0
    return w


@pytest.mark.parametrize("name", ["qubit_couple_rot_e5", "qubit_couple_rot_e1_nores",
                                  "qubit_hyperfine", "qubit_couple_rot_nh", "qubit_t1_0K_rot",
                                  "qubit_t1_mK_rot_e2"])
def test_batch_rotating_matches_reference_output(name):
    """Reference runs in the rotating frame (CF6:5 and CF2:1, residual and
    plain arithmetic, a hyperfine pair, the complex non-Hermitian basis,
    decay -- damped e^{L0 h} blocks -- at K = 1 and 2):
    the batched kernel's full-state trace against the reference's
    densities."""
    from superspinsim_gb300.generate_simulator import number_of_samples, unflatten_density
    from superspinsim_gb300.sweep import Sweep
    c = load_case(name)
    vm = c["vectorisation_map"] if bool(c.get("meta_herm", True)) else None
    K, F, res = int(c["meta_K"]), int(c["meta_F"]), bool(c["meta_res"])
    t0, tf, dt = (float(v) for v in c["times"])
    T = number_of_samples(t0, tf, dt)
    sw = Sweep(c["generators"], vm, number_of_exponentials=K, number_of_fine_divisions=F,
               use_rotating=True, time_step=dt, use_residual=res)
    flat = sw.flatten(c["rho0"][None])
    _, fin, tr = sw.plan.batch(flat, c["program"][None], t0, dt, T, F, want_final=True,
                               want_trace=True)
    d = unflatten_density(tr[0], c["rho0"].shape[0], vm)
    # plain (non-residual) reference arithmetic adds the identity before its
    # squarings and loses the small diagonal terms: 1e-9, as for the dense
    # path's Taylor exponential
    assert np.abs(d - c["density"]).max() <= (1e-11 if res else 1e-9)
    assert np.array_equal(fin[0], tr[0, -1])


def test_batch_rotating_odmr_against_oracle():
    """NV-7 ODMR in the rotating frame: readouts and final states against the
    oracle's rotating vector mode, and the readout against the lab frame
    (the two frames integrate the same equation to within 1e-9)."""
    from superspinsim_gb300.rotating import make_rotating
    from superspinsim_gb300.sweep import Sweep
    c = load_case("nv7_n49")
    gens, vm = c["generators"], c["vectorisation_map"]
    N = vm.shape[0]
    freqs = F_RES + np.linspace(-30e6, 30e6, 6)
    progs = _odmr_programs(freqs, 5e6/28.025e9, 10/65.9)
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    flat = np.stack([oracle.flatten(rho, vm, N)]*len(freqs))
    T, dt, F = 4, 1e-9, 200
    w = _excited_weights(vm)
    sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F,
               use_rotating=True, time_step=dt)
    ro, fin = sw.plan.batch(flat, progs, 0.0, dt, T, F, readout_weights=w, want_final=True)
    info = sw.info()
    assert info["rows"] == 19 and info["degree"] < 8
    new, V, Vi, d, s = make_rotating(gens[0], list(gens[1:]))
    W, nodes = quadrature(2)
    rot = dict(generators_rotating=np.array(new), vectors_real=V, inv_vectors_real=Vi,
               doubles=np.asarray(d).reshape(-1, 2), singles=s)
    _, ref = oracle.simulate(gens, np.stack([rho]*len(freqs)), 0.0, T*dt + 1e-13, dt, progs,
                             K=2, W=W, nodes=nodes, F=F, vectorisation_map=vm, rotating=rot,
                             mode="vector", degree=16, flat_out=True)
    assert np.abs(fin - ref[:, -1]).max() <= 1e-12
    assert np.abs(ro - ref @ w).max() <= 1e-12
    lab = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F)
    ro_lab, _ = lab.plan.batch(flat, progs, 0.0, dt, T, F, readout_weights=w)
    assert np.abs(ro - ro_lab).max() <= 1e-9


def test_batch_rotating_uneven_chunked_and_resumed(tmp_path):
    """Ramsey protocol with uneven lengths in the rotating frame: chunked
    launches and a resumed run agree with the one-shot run to rounding (a
    chunk hands its state over in the lab basis, V x, and the next one
    starts from V^-1 of it), and the one-shot run matches the oracle
    trajectory by trajectory."""
    pytest.importorskip("torch")
    from superspinsim_gb300 import protocols
    from superspinsim_gb300.rotating import make_rotating
    from superspinsim_gb300.sweep import ChunkedRun, Sweep, population_weights
    c = load_case("nv7_n49")
    gens, vm = c["generators"], c["vectorisation_map"]
    rng = np.random.default_rng(21)
    B = 7
    progs, dur = protocols.ramsey(rng.uniform(20e6, 60e6, B), rng.uniform(-5e6, 5e6, B),
                                  rng.uniform(0, 20e-9, B), F_RES, 10/65.9, t_init=10e-9,
                                  t_read=5e-9)
    dt, F = 1e-9, 40
    samples = np.ceil(dur/dt).astype(np.int32)
    T = int(samples.max())
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    w = population_weights(vm, [3, 4, 5])
    sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F,
               use_rotating=True, time_step=dt)
    one = sw.run(np.repeat(rho[None], B, axis=0), progs, 0.0, T*dt + 1e-13, dt, samples=samples,
                 readout_weights=w, final_state=True)
    run = ChunkedRun(sw, rho, progs, 0.0, dt, T, samples=samples, readout_weights=w).run(chunk=4)
    r = run.results()
    assert np.abs(r["readout"] - one["readout"]).max() <= 1e-13
    assert np.abs(r["final"] - one["final"]).max() <= 1e-13
    half = ChunkedRun(sw, rho, progs, 0.0, dt, T, samples=samples, readout_weights=w)
    half.step(T//2)
    half.save(tmp_path/"ck.npz")
    resumed = ChunkedRun(sw, rho, progs, 0.0, dt, T, samples=samples, readout_weights=w)
    resumed.load(tmp_path/"ck.npz").run(chunk=5)
    assert np.abs(resumed.results()["readout"] - one["readout"]).max() <= 1e-13
    new, V, Vi, d, s = make_rotating(gens[0], list(gens[1:]))
    W, nodes = quadrature(2)
    rot = dict(generators_rotating=np.array(new), vectors_real=V, inv_vectors_real=Vi,
               doubles=np.asarray(d).reshape(-1, 2), singles=s)
    for b in range(B):
        n = int(samples[b])
        _, ref = oracle.simulate(gens, rho, 0.0, n*dt + 1e-13, dt, progs[b], K=2, W=W,
                                 nodes=nodes, F=F, vectorisation_map=vm, rotating=rot,
                                 mode="vector", degree=16, flat_out=True)
        assert np.abs(one["readout"][b, :n] - ref @ w).max() <= 1e-12
        assert np.abs(one["final"][b] - ref[-1]).max() <= 1e-12


def test_batch_rotating_needs_row_parts():
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.sweep import Sweep
    c = load_case("nv7_n49")
    sw = Sweep(c["generators"], c["vectorisation_map"], number_of_exponentials=2,
               number_of_fine_divisions=10, use_rotating=True, time_step=1e-9, variant=1)
    progs = _odmr_programs([F_RES], 5e6/28.025e9, 10/65.9)
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    with pytest.raises(_lib.SSSError, match="row-part"):
        sw.run(rho, progs, 0.0, 2e-9 + 1e-13, 1e-9, final_state=True)


def test_batch_rotating_ragged_with_empty_trajectories():
    """Ragged lengths including trajectories of zero samples, rotating frame:
    the batched readouts and final states against the plain path on the same
    rotating plan; an empty trajectory's final state is its initial state (to
    the rounding of V V^-1) and its readout row stays zero."""
    from superspinsim_gb300.sweep import Sweep
    c = load_case("nv7_n49")
    gens, vm = c["generators"], c["vectorisation_map"]
    N = vm.shape[0]
    rng = np.random.default_rng(8)
    B, T, dt, F = 13, 5, 1e-9, 40
    progs = _odmr_programs(F_RES + rng.uniform(-5e6, 5e6, B), 5e6/28.025e9, 10/65.9)
    samples = rng.integers(0, T + 1, B).astype(np.int32)
    samples[[0, 5]] = 0
    rho = np.zeros((7, 7), complex)
    rho[0, 0], rho[1, 1] = 0.4, 0.6
    flat = np.stack([oracle.flatten(rho, vm, N)]*B)
    w = _excited_weights(vm)
    sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F,
               use_rotating=True, time_step=dt)
    ro, fin = sw.plan.batch(flat, progs, 0.0, dt, T, F, samples=samples, readout_weights=w,
                            want_final=True)
    full = sw.plan.simulate(flat, progs, 0.0, dt, T, F)   # plain path, same rotating plan
    for b in range(B):
        n = int(samples[b])
        if n:
            assert np.abs(ro[b, :n] - full[b, :n] @ w).max() <= 1e-12
        assert np.all(ro[b, n:] == 0.0)
        last = full[b, n - 1] if n else flat[b]
        assert np.abs(fin[b] - last).max() <= 1e-12
