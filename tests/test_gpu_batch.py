"""Batched persistent kernel (sss_batch_run through the C-ABI) against the
oracle, on the 7-level NV model of the reference's own generators."""
import numpy as np
import pytest

from conftest import load_case, quadrature
from oracle import oracle

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("name", ["nv7_n49", "nv7_n19"])
@pytest.mark.parametrize("lanes,variant", [(0, 0), (1, 0), (4, 0), (32, 0), (0, 1), (16, 1),
                                           (0, 2), (8, 2), (0, 3), (32, 3), (0, 4), (8, 4),
                                           (16, 4), (32, 4), (64, 4), (128, 4), (0, 6), (8, 6),
                                           (16, 6), (32, 6), (64, 6), (128, 6), (0, 7), (8, 7),
                                           (16, 7), (32, 7)])
def test_batch_odmr_against_oracle(name, lanes, variant):
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.quadratures import method
    c = load_case(name)
    vm = c["vectorisation_map"]
    N = vm.shape[0]
    f_res = 2.870e9 + 28.025e9*5e-3
    freqs = f_res + np.linspace(-30e6, 30e6, 6)
    progs = _odmr_programs(freqs, 5e6/28.025e9, 10/65.9)
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    rho0 = np.stack([oracle.flatten(rho, vm, N)]*len(freqs))
    W, nodes = method(2)
    T, dt, F = 4, 1e-9, 200
    plan = _lib.Plan(c["generators"], W, nodes)
    plan.set_batch_config(lanes=lanes, variant=variant)
    w = _excited_weights(vm)
    ro, fin = plan.batch(rho0, progs, 0.0, dt, T, F, readout_weights=w, want_final=True)
    info = plan.batch_info()
    assert info["rows"] == (19 if True else N)
    _, ref = oracle.simulate(c["generators"], np.stack([rho]*len(freqs)), 0.0,
                             T*dt + 1e-13, dt, progs, K=2, W=W, nodes=nodes, F=F,
                             vectorisation_map=vm, mode="vector", degree=16,
                             flat_out=True)
    assert np.abs(fin - ref[:, -1]).max() <= 1e-12
    assert np.abs(ro - ref @ w).max() <= 1e-12


@pytest.mark.parametrize("lanes,variant", [(0, 0), (0, 4), (64, 4), (0, 6), (16, 6), (0, 7),
                                           (32, 7)])
def test_batch_uneven_lengths_and_plain_agree(lanes, variant):
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.quadratures import method
    c = load_case("nv7_n49")
    vm = c["vectorisation_map"]
    N = vm.shape[0]
    rng = np.random.default_rng(7)
    B, T, dt, F = 37, 6, 1e-9, 50
    f_res = 2.870e9 + 28.025e9*5e-3
    progs = _odmr_programs(f_res + rng.uniform(-5e6, 5e6, B), 5e6/28.025e9, 10/65.9)
    samples = rng.integers(0, T + 1, B).astype(np.int32)
    rho = np.zeros((7, 7), complex)
    rho[0, 0] = 0.5
    rho[1, 1] = 0.5
    rho0 = np.stack([oracle.flatten(rho, vm, N)]*B)
    W, nodes = method(2)
    plan = _lib.Plan(c["generators"], W, nodes)
    plan.set_batch_config(lanes=lanes, variant=variant)
    w = _excited_weights(vm)
    ro, fin = plan.batch(rho0, progs, 0.0, dt, T, F, samples=samples, readout_weights=w,
                         want_final=True)
    full = plan.simulate(rho0, progs, 0.0, dt, T, F)   # plain path, all T samples
    for b in range(B):
        n = samples[b]
        if n > 0:
            assert np.abs(ro[b, :n] - full[b, :n] @ w).max() <= 1e-12
        assert np.all(ro[b, n:] == 0.0)
        last = full[b, n - 1] if n > 0 else rho0[b]
        assert np.abs(fin[b] - last).max() <= 1e-12


def test_batch_empty_and_zero_state():
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.quadratures import method
    c = load_case("nv7_n19")
    W, nodes = method(2)
    plan = _lib.Plan(c["generators"], W, nodes)
    N = c["generators"].shape[1]
    progs = _odmr_programs([3e9], 1e-4, 0.1)
    ro, fin = plan.batch(np.zeros((1, N)), progs, 0.0, 1e-9, 3, 10,
                         readout_weights=np.ones(N), want_final=True)
    assert np.all(ro == 0) and np.all(fin == 0)
    ro, fin = plan.batch(np.zeros((0, N)), progs[:0], 0.0, 1e-9, 3, 10,
                         readout_weights=np.ones(N), want_final=True)
    assert ro.shape == (0, 3)


@pytest.mark.parametrize("lanes,variant", [(0, 0), (16, 4), (32, 4), (8, 6), (16, 6), (0, 6),
                                           (8, 7), (16, 7), (32, 7)])
def test_batch_ramsey_uneven_against_oracle(lanes, variant):
    """Uneven Ramsey protocol (laser init, pi/2 - tau - pi/2, laser readout)
    with per-trajectory lengths, against the oracle trajectory by trajectory."""
    from superspinsim_gb300 import _lib, protocols
    from superspinsim_gb300.quadratures import method
    c = load_case("nv7_n19")
    vm = c["vectorisation_map"]
    N = vm.shape[0]
    rng = np.random.default_rng(11)
    B = 9
    f_res = 2.870e9 + 28.025e9*5e-3
    rabi = rng.uniform(20e6, 60e6, B)
    det = rng.uniform(-5e6, 5e6, B)
    tau = rng.uniform(0, 30e-9, B)
    progs, dur = protocols.ramsey(rabi, det, tau, f_res, 10/65.9, t_init=20e-9, t_read=10e-9)
    dt, F = 1e-9, 40
    samples = np.ceil(dur/dt).astype(np.int32)
    T = int(samples.max())
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    rho0 = np.stack([oracle.flatten(rho, vm, N)]*B)
    W, nodes = method(2)
    plan = _lib.Plan(c["generators"], W, nodes)
    plan.set_batch_config(lanes=lanes, variant=variant, cta_threads=64)
    w = _excited_weights(vm)
    ro, fin = plan.batch(rho0, progs, 0.0, dt, T, F, samples=samples, readout_weights=w,
                         want_final=True)
    for b in range(B):
        n = int(samples[b])
        _, ref = oracle.simulate(c["generators"], rho, 0.0, n*dt + 1e-13, dt, progs[b], K=2,
                                 W=W, nodes=nodes, F=F, vectorisation_map=vm, mode="vector",
                                 degree=16, flat_out=True)
        assert np.abs(ro[b, :n] - ref @ w).max() <= 1e-12
        assert np.abs(fin[b] - ref[-1]).max() <= 1e-12


@pytest.mark.parametrize("lanes,variant", [(0, 0), (32, 1), (128, 4), (256, 4), (128, 6),
                                           (256, 6)])
def test_batch_nv21_against_oracle(lanes, variant):
    """21-level NV with 14N (441 x 441), 4 ODMR trajectories: the register
    kernel and the row-part kernel with groups of 4 and 8 warps (one
    trajectory per CTA)."""
    from superspinsim_gb300 import _lib, protocols
    from superspinsim_gb300.quadratures import method
    c = load_case("nv21_n441")
    gens, vm = c["generators"], c["vectorisation_map"]
    N = vm.shape[0]
    f_res = 2.870e9 + 28.025e9*0.05
    progs = protocols.odmr(f_res + np.array([-3e6, -1e6, 1e6, 3e6]), 5e6, 10/65.9)
    rho = np.zeros((21, 21), complex)
    for k in range(3, 6):
        rho[k, k] = 1/3    # ms = 0 with the nitrogen spin mixed
    rho0 = np.stack([oracle.flatten(rho, vm, N)]*4)
    W, nodes = method(2)
    T, dt, F = 2, 1e-9, 50
    plan = _lib.Plan(gens, W, nodes)
    plan.set_batch_config(lanes=lanes, variant=variant)
    ro, fin = plan.batch(rho0, progs, 0.0, dt, T, F, want_final=True)
    info = plan.batch_info()
    assert info["rows"] < N
    if lanes:
        assert info["lanes"] == lanes
    # at 32 lanes the row parts of 1,475 entries do not fit one warp
    plan2 = _lib.Plan(gens, W, nodes)
    plan2.set_batch_config(lanes=32, variant=4)
    with pytest.raises(_lib.SSSError, match="row-part"):
        plan2.batch(rho0, progs, 0.0, dt, T, F, want_final=True)
    _, ref = oracle.simulate(gens, np.stack([rho]*4), 0.0, T*dt + 1e-13, dt, progs, K=2, W=W,
                             nodes=nodes, F=F, vectorisation_map=vm, mode="vector", degree=16,
                             flat_out=True)
    assert np.abs(fin - ref[:, -1]).max() <= 1e-12


@pytest.mark.parametrize("variant", [0, 4, 6, 7])
def test_chunked_runs_graph_replay_and_resume(tmp_path, variant):
    """Prepare once, launch in chunks: identical to the one-shot run; the
    chunk sequence captured in a CUDA graph replays to the same result; a
    run saved half-way and resumed finishes identically."""
    torch = pytest.importorskip("torch")
    from superspinsim_gb300 import protocols
    from superspinsim_gb300.sweep import ChunkedRun, Sweep, population_weights
    c = load_case("nv7_n49")
    vm = c["vectorisation_map"]
    f_res = 2.870e9 + 28.025e9*5e-3
    rng = np.random.default_rng(3)
    B = 40
    progs, dur = protocols.ramsey(rng.uniform(20e6, 60e6, B), rng.uniform(-5e6, 5e6, B),
                                  rng.uniform(0, 20e-9, B), f_res, 10/65.9, t_init=10e-9,
                                  t_read=5e-9)
    dt = 1e-9
    samples = np.ceil(dur/dt).astype(np.int32)
    T = int(samples.max())
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    w = population_weights(vm, [3, 4, 5])
    sw = Sweep(c["generators"], vm, number_of_exponentials=2, number_of_fine_divisions=20)
    sw.plan.set_batch_config(variant=variant)
    one = sw.run(np.repeat(rho[None], B, axis=0), progs, 0.0, T*dt + 1e-13, dt, samples=samples,
                 readout_weights=w, final_state=True)
    run = ChunkedRun(sw, rho, progs, 0.0, dt, T, samples=samples, readout_weights=w).run(chunk=3)
    r = run.results()
    assert np.array_equal(r["readout"], one["readout"])
    assert np.array_equal(r["final"], one["final"])
    g = ChunkedRun(sw, rho, progs, 0.0, dt, T, samples=samples, readout_weights=w)
    g.capture(chunk=4).replay()
    torch.cuda.synchronize()
    r2 = g.results()
    assert np.array_equal(r2["readout"], one["readout"])
    assert np.array_equal(r2["final"], one["final"])
    half = ChunkedRun(sw, rho, progs, 0.0, dt, T, samples=samples, readout_weights=w)
    half.step(T//2)
    half.save(tmp_path/"ck.npz")
    resumed = ChunkedRun(sw, rho, progs, 0.0, dt, T, samples=samples, readout_weights=w)
    resumed.load(tmp_path/"ck.npz").run(chunk=5)
    r3 = resumed.results()
    assert np.array_equal(r3["readout"], one["readout"])
    assert np.array_equal(r3["final"], one["final"])


@pytest.mark.parametrize("name", ["coherent_chain", "hbn_bell"])
@pytest.mark.parametrize("variant", [0, 4, 7])
def test_batch_coupled_blocks_against_oracle(name, variant):
    """Systems with coherent block couplings (Vc in L0, Vr in Gr, scaled by
    the fourth channel) and with Bell-state couplings through the batched
    kernel: a sweep over the drive frequency and the fourth channel's
    level, final states and readouts against the oracle."""
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.quadratures import method
    c = load_case(name)
    vm = c["vectorisation_map"]
    N = vm.shape[0]
    B = 8
    progs = np.repeat(c["program"][None], B, axis=0)
    progs[:, 0, 0, 3] *= np.linspace(0.9, 1.1, B)
    progs[:, 3, 0, 0] = 1.0
    progs[:, 3, 0, 1] = np.linspace(0.0, 1.0, B)
    rho0 = np.stack([oracle.flatten(c["rho0"], vm, N)]*B)
    w = np.array([1.0 if y == x and ch == 0 else 0.0 for y, x, ch in vm])
    w[0] = 2.0
    W, nodes = method(2)
    T, dt, F = 4, 1e-9, 20
    plan = _lib.Plan(c["generators"], W, nodes)
    plan.set_batch_config(variant=variant)
    ro, fin = plan.batch(rho0, progs, 0.0, dt, T, F, readout_weights=w, want_final=True)
    _, ref = oracle.simulate(c["generators"], np.stack([c["rho0"]]*B), 0.0, T*dt + 1e-13, dt,
                             progs, K=2, W=W, nodes=nodes, F=F, vectorisation_map=vm,
                             mode="vector", degree=16, flat_out=True)
    assert np.abs(fin - ref[:, -1]).max() <= 1e-12
    assert np.abs(ro - ref @ w).max() <= 1e-12
    if name == "coherent_chain":
        # the second qubit (levels 5, 6) is reached only through the Vr
        # coupling: empty at level 0 of the fourth channel, filled at 1
        q2 = [k for k, (y, x, ch) in enumerate(vm) if y == x and y in (5, 6) and ch == 0]
        assert np.abs(fin[0, q2]).max() <= 1e-15 and fin[-1, q2].sum() > 1e-4


@pytest.mark.parametrize("name,lanes,variant", [("nv7_n49", 32, 7), ("nv7_n49", 16, 6),
                                                ("nv21_n441", 128, 6)])
def test_bank_placement_reports_fewer_conflicts(name, lanes, variant):
    """A slot-programmed run reports the modelled extra shared-memory
    wavefronts per Horner term before and after the bank-aware placement;
    the placement never makes them worse, and a second run of the same
    batch reuses the cached placement (same figures, same results)."""
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.quadratures import method
    c = load_case(name)
    vm = c["vectorisation_map"]
    N = vm.shape[0]
    n = 7 if name == "nv7_n49" else 21
    rho = np.zeros((n, n), complex)
    for k in ((1,) if n == 7 else (3, 4, 5)):
        rho[k, k] = 1.0/(1 if n == 7 else 3)
    B = 4
    f0 = 2.870e9 + 28.025e9*(5e-3 if n == 7 else 0.05)
    progs = _odmr_programs(f0 + np.linspace(-5e6, 5e6, B), 5e6/28.025e9, 10/65.9)
    rho0 = np.stack([oracle.flatten(rho, vm, N)]*B)
    W, nodes = method(2)
    plan = _lib.Plan(c["generators"], W, nodes)
    plan.set_batch_config(lanes=lanes, variant=variant)
    _, f1 = plan.batch(rho0, progs, 0.0, 1e-9, 2, 20, want_final=True)
    b1 = plan.batch_info()["bank_extra_wavefronts_per_term"]
    _, f2 = plan.batch(rho0, progs, 0.0, 1e-9, 2, 20, want_final=True)
    b2 = plan.batch_info()["bank_extra_wavefronts_per_term"]
    assert 0 <= b1["renumbered"] <= b1["lane_order"]
    assert b1 == b2 and np.array_equal(f1, f2)
    if name == "nv21_n441":
        assert b1["renumbered"] * 4 <= b1["lane_order"]


def test_autotuner_picks_a_working_configuration():
    pytest.importorskip("torch")
    from superspinsim_gb300 import protocols
    from superspinsim_gb300.sweep import Sweep, population_weights
    from superspinsim_gb300.tune import autotune
    c = load_case("nv7_n19")
    vm = c["vectorisation_map"]
    progs = protocols.odmr(2.870e9 + 28.025e9*5e-3 + np.linspace(-5e6, 5e6, 24), 5e6, 0.15)
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    sw = Sweep(c["generators"], vm, number_of_exponentials=2, number_of_fine_divisions=20)
    res = autotune(sw, rho, progs, 1e-9, probe_samples=1, repeats=1)
    assert len([t for t in res["trials"] if "ms" in t]) >= 2
    w = population_weights(vm, [3, 4, 5])
    out = sw.run(rho, progs, 0.0, 3e-9 + 1e-13, 1e-9, readout_weights=w, final_state=True)
    sw2 = Sweep(c["generators"], vm, number_of_exponentials=2, number_of_fine_divisions=20)
    out2 = sw2.run(rho, progs, 0.0, 3e-9 + 1e-13, 1e-9, readout_weights=w, final_state=True)
    assert np.abs(out["final"] - out2["final"]).max() <= 1e-13


def test_autotuner_times_launch_lengths():
    """The launch-length stage times a 16-sample window as 16, 4 and 1
    launches for the chosen configuration, picks the shortest launch within
    the tolerance of the fastest, and a ChunkedRun with no chunk length
    uses it; the chunked result equals a single launch bit for bit."""
    pytest.importorskip("torch")
    from superspinsim_gb300 import protocols
    from superspinsim_gb300.sweep import ChunkedRun, Sweep, population_weights
    from superspinsim_gb300.tune import autotune
    c = load_case("nv7_n49")
    vm = c["vectorisation_map"]
    progs = protocols.odmr(2.870e9 + 28.025e9*5e-3 + np.linspace(-5e6, 5e6, 40), 5e6, 0.15)
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    sw = Sweep(c["generators"], vm, number_of_exponentials=2, number_of_fine_divisions=10)
    res = autotune(sw, rho, progs, 1e-9, probe_samples=1, repeats=1, lanes=(0, 32),
                   variants=(4, 7), threads=(32,), chunks=(1, 4, 16), use_cache=False)
    trials = res["chunk_trials"]
    assert [t["launches"] for t in trials] == [16, 4, 1]
    best = min(t["ms"] for t in trials)
    c_pick = res["samples_per_launch"]
    assert c_pick in (1, 4, 16) and sw.tuned_chunk == c_pick
    assert next(t for t in trials if t["samples_per_launch"] == c_pick)["ms"] <= best*1.01
    w = population_weights(vm, [3, 4, 5])
    T = 12
    tuned = ChunkedRun(sw, rho, progs, 0.0, 1e-9, T, readout_weights=w).run().results()
    whole = ChunkedRun(sw, rho, progs, 0.0, 1e-9, T, readout_weights=w).run(chunk=T).results()
    assert np.array_equal(tuned["readout"], whole["readout"])
    assert np.array_equal(tuned["final"], whole["final"])


def test_dropin_simulate_nv21_uses_batched_trace():
    """generate_simulator/simulate at N = 441 (beyond the dense plain path)
    runs the batched kernel with a full-state trace; against the oracle."""
    from superspinsim_gb300 import generate_simulator, protocols
    from superspinsim_gb300.quadratures import method
    c = load_case("nv21_n441")
    gens, vm = c["generators"], c["vectorisation_map"]
    f_res = 2.870e9 + 28.025e9*0.05
    prog = protocols.odmr([f_res + 2e6], 5e6, 10/65.9)[0]
    rho = np.zeros((21, 21), complex)
    for k in range(3, 6):
        rho[k, k] = 1/3
    sim = generate_simulator(prog, gens, vm, number_of_exponentials=2,
                             number_of_fine_divisions=50)
    t, d = sim(rho, 0.0, 3e-9 + 1e-13, 1e-9)
    W, nodes = method(2)
    _, ref = oracle.simulate(gens, rho, 0.0, 3e-9 + 1e-13, 1e-9, prog, K=2, W=W, nodes=nodes,
                             F=50, vectorisation_map=vm, mode="vector", degree=16)
    assert d.shape == (3, 21, 21)
    assert np.abs(d - ref).max() <= 1e-12


def test_phased_uneven_batch_chunked_graph_and_oracle():
    """3000 short uneven Ramsey trajectories: enough for the automatic lanes
    to widen in phases as trajectories finish (16 lanes, then 32 and wider).
    The one-shot run, a chunked run and its CUDA-graph capture -- all
    prepared with the sample counts -- agree bit for bit (the same layout
    at every output sample), and sampled trajectories match the oracle."""
    torch = pytest.importorskip("torch")
    from superspinsim_gb300 import protocols
    from superspinsim_gb300.sweep import ChunkedRun, Sweep, population_weights
    c = load_case("nv7_n49")
    gens, vm = c["generators"], c["vectorisation_map"]
    f_res = 2.870e9 + 28.025e9*5e-3
    rng = np.random.default_rng(11)
    B = 3000
    progs, dur = protocols.ramsey(rng.uniform(40e6, 80e6, B), rng.uniform(-5e6, 5e6, B),
                                  rng.uniform(0, 30e-9, B), f_res, 10/65.9, t_init=4e-9,
                                  t_read=3e-9)
    dt, F = 1e-9, 10
    samples = np.ceil(dur/dt).astype(np.int32)
    T = int(samples.max())
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    w = population_weights(vm, [3, 4, 5])
    sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F)
    one = sw.run(rho, progs, 0.0, T*dt + 1e-13, dt, samples=samples, readout_weights=w,
                 final_state=True)
    assert sw.plan.last_launches() >= 3     # three lane counts, at least
    run = ChunkedRun(sw, rho, progs, 0.0, dt, T, samples=samples, readout_weights=w).run(chunk=7)
    r = run.results()
    assert np.array_equal(r["readout"], one["readout"])
    assert np.array_equal(r["final"], one["final"])
    g = ChunkedRun(sw, rho, progs, 0.0, dt, T, samples=samples, readout_weights=w)
    g.capture(chunk=9).replay()
    torch.cuda.synchronize()
    r2 = g.results()
    assert np.array_equal(r2["readout"], one["readout"])
    assert np.array_equal(r2["final"], one["final"])
    W, nodes = quadrature(2)
    order = np.argsort(samples)
    for b in (order[0], order[B//2], order[-1], 17):
        n = int(samples[b])
        _, ref = oracle.simulate(gens, rho, 0.0, n*dt + 1e-13, dt, progs[b], K=2, W=W,
                                 nodes=nodes, F=F, vectorisation_map=vm, mode="vector",
                                 degree=16, flat_out=True)
        assert np.abs(one["final"][b] - ref[-1]).max() <= 1e-12
        assert np.abs(one["readout"][b, :n] - ref @ w).max() <= 1e-12
        assert np.all(one["readout"][b, n:] == 0.0)


def test_register_state_variant_matches_row_parts():
    """Variant 5 (the row-part layout with the state in registers, moved by
    warp shuffles) against variant 4 (state in shared memory): the same
    arithmetic in the same order, so the same numbers (up to the sign of a
    zero) -- on a uniform NV-7 sweep, an uneven phased batch and a table
    run -- and the oracle."""
    from superspinsim_gb300 import protocols
    from superspinsim_gb300.sweep import Sweep, population_weights
    c = load_case("nv7_n49")
    gens, vm = c["generators"], c["vectorisation_map"]
    f_res = 2.870e9 + 28.025e9*5e-3
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    w = population_weights(vm, [3, 4, 5])
    dt, F = 1e-9, 40
    freqs = f_res + np.linspace(-20e6, 20e6, 300)
    progs = np.zeros((len(freqs), 4, 1, 5))
    progs[:, :, :, 0] = np.inf
    progs[:, 0, 0, 2] = 5e6/28.025e9
    progs[:, 0, 0, 3] = freqs
    progs[:, 3, 0, 1] = 10/65.9
    rng = np.random.default_rng(4)
    B = 2600
    rprogs, dur = protocols.ramsey(rng.uniform(40e6, 80e6, B), rng.uniform(-5e6, 5e6, B),
                                   rng.uniform(0, 20e-9, B), f_res, 10/65.9, t_init=4e-9,
                                   t_read=3e-9)
    samples = np.ceil(dur/dt).astype(np.int32)
    Tr = int(samples.max())
    out = {}
    for variant in (4, 5):
        sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F,
                   variant=variant)
        a = sw.run(rho, progs, 0.0, 6*dt + 1e-13, dt, readout_weights=w, final_state=True)
        assert sw.info()["lanes"] == 32
        b = sw.run(rho, rprogs, 0.0, Tr*dt + 1e-13, dt, samples=samples, readout_weights=w,
                   final_state=True)
        out[variant] = (a, b)
    for k in ("readout", "final"):
        assert np.array_equal(out[4][0][k], out[5][0][k])
        assert np.array_equal(out[4][1][k], out[5][1][k])
    a = out[5][0]
    W, nodes = quadrature(2)
    _, ref = oracle.simulate(gens, np.stack([rho]*3), 0.0, 6*dt + 1e-13, dt, progs[[0, 150, 299]],
                             K=2, W=W, nodes=nodes, F=F, vectorisation_map=vm, mode="vector",
                             degree=16, flat_out=True)
    assert np.abs(a["final"][[0, 150, 299]] - ref[:, -1]).max() <= 1e-12
    assert np.abs(a["readout"][[0, 150, 299]] - ref @ w).max() <= 1e-12
