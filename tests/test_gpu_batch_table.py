"""Batched runs from a coefficient table (sss_batch_run_table): the fallback
for arbitrary sampler callables, against the same runs from programs,
against the oracle and against the plain path on the same table."""
import math

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


def _sampler(prog, lab=True):
    """The reference's sampler form: write the row at time t in place."""
    from superspinsim_gb300.program import array_value

    def sampler(time, row):
        if lab:
            row[0] = 1.0
        for ch in range(4):
            row[ch + (1 if lab else 0)] = array_value(prog, ch, time)
    return sampler


def _nv7():
    c = load_case("nv7_n49")
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    return c["generators"], c["vectorisation_map"], rho


@pytest.mark.parametrize("rotating", [False, True], ids=["lab", "rotating"])
def test_table_run_matches_programs_and_oracle(rotating):
    """Six NV-7 ODMR trajectories of uneven length, sampled on the host by
    sampler callables: readouts and final states equal the program run's
    (the coefficients differ only by host versus device cosine rounding)
    and the oracle's vector mode."""
    from superspinsim_gb300.sweep import Sweep, population_weights
    gens, vm, rho = _nv7()
    B, T, dt, F = 6, 4, 1e-9, 100
    progs = _odmr_programs(F_RES + np.linspace(-20e6, 20e6, B), 5e6/28.025e9, 10/65.9)
    samples = np.array([4, 1, 3, 0, 4, 2], dtype=np.int32)
    w = population_weights(vm, [3, 4, 5])
    sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F,
               use_rotating=rotating, time_step=dt)
    tf = T*dt + 1e-13
    a = sw.run(rho, progs, 0.0, tf, dt, samples=samples, readout_weights=w, final_state=True)
    samplers = [_sampler(p, lab=not rotating) for p in progs]
    b = sw.run(rho, samplers, 0.0, tf, dt, samples=samples, readout_weights=w, final_state=True)
    assert np.abs(a["readout"] - b["readout"]).max() <= 1e-13
    assert np.abs(a["final"] - b["final"]).max() <= 1e-13
    assert np.all(b["readout"][np.arange(T)[None, :] >= samples[:, None]] == 0.0)
    W, nodes = quadrature(2)
    rot = None
    if rotating:
        from superspinsim_gb300.rotating import make_rotating
        new, V, Vi, d, s = make_rotating(gens[0], list(gens[1:]))
        rot = dict(generators_rotating=np.array(new), vectors_real=V, inv_vectors_real=Vi,
                   doubles=np.asarray(d).reshape(-1, 2), singles=s)
    for k in range(B):
        n = int(samples[k])
        if n == 0:
            assert np.abs(b["final"][k] - oracle.flatten(rho, vm, vm.shape[0])).max() <= 1e-14
            continue
        _, ref = oracle.simulate(gens, rho, 0.0, n*dt + 1e-13, dt, progs[k], K=2, W=W,
                                 nodes=nodes, F=F, vectorisation_map=vm, rotating=rot,
                                 mode="vector", degree=16, flat_out=True)
        assert np.abs(b["final"][k] - ref[-1]).max() <= 1e-12
        assert np.abs(b["readout"][k, :n] - ref @ w).max() <= 1e-12


def test_table_with_varying_L0_coefficient_against_plain_path():
    """A table whose L0 column varies in time (not folded into the constant
    part of Omega, so L0 is assembled every step like a drive) and whose
    y field is non-zero: the batched table run against the plain path
    (sss_simulate) on the same table."""
    from superspinsim_gb300 import _lib
    gens, vm, rho = _nv7()
    N = vm.shape[0]
    W, nodes = quadrature(2)
    plan = _lib.Plan(gens, W, nodes)
    B, T, dt, F = 3, 3, 1e-9, 50
    Q, G = len(nodes), gens.shape[0]
    tab = np.zeros((B, F, T, Q, G))
    for b in range(B):
        f = F_RES + 7e6*(b - 1)
        for r in range(F):
            for t in range(T):
                for k in range(Q):
                    tn = ((0.0 + (r*dt)/F) + dt*t) + (dt*nodes[k])/F
                    tab[b, r, t, k] = [1.0 + 0.05*math.sin(2*math.pi*1e8*tn),
                                       2e-4*math.cos(2*math.pi*f*tn),
                                       1e-4*math.sin(2*math.pi*f*tn), 0.0, 10/65.9]
    tab = tab.reshape(B, F*T*Q, G)
    flat = np.stack([oracle.flatten(rho, vm, N)]*B)
    ref = plan.simulate(flat, None, 0.0, dt, T, F, table=tab)
    _, fin, tr = plan.batch(flat, None, 0.0, dt, T, F, want_final=True, want_trace=True,
                            table=tab)
    assert np.abs(tr - ref).max() <= 1e-12
    assert np.array_equal(fin, tr[:, -1])


def test_nv21_dropin_with_sampler_callable():
    """The drop-in above the dense path's size (NV-21, N = 441) with the
    reference's sampler form: equal to the same simulator built on the
    equivalent program."""
    import argparse
    import bench
    from superspinsim_gb300 import generate_simulator
    args = argparse.Namespace(n_traj=2, duration=bench.DURATION)
    gens, vm, progs, rho, _, _, _, _ = bench.build_workload("nv21", args)
    prog = progs[1]
    kw = dict(number_of_exponentials=2, number_of_fine_divisions=200)
    s1 = generate_simulator(prog, gens, vm, **kw)
    s2 = generate_simulator(_sampler(prog), gens, vm, **kw)
    t1, d1 = s1(rho, 0.0, 2e-9 + 1e-13, 1e-9)
    t2, d2 = s2(rho, 0.0, 2e-9 + 1e-13, 1e-9)
    assert d1.shape == (2, 21, 21) and np.array_equal(t1, t2)
    assert np.abs(d1 - d2).max() <= 1e-13


def test_table_errors():
    from superspinsim_gb300 import _lib
    gens, vm, rho = _nv7()
    N = vm.shape[0]
    W, nodes = quadrature(2)
    plan = _lib.Plan(gens, W, nodes)
    T, F = 2, 10
    flat = oracle.flatten(rho, vm, N)[None]
    tab = np.zeros((1, F*T*len(nodes), gens.shape[0]))
    tab[:, :, 0] = 1.0
    with pytest.raises(ValueError, match="coefficient table"):
        plan.batch(flat, None, 0.0, 1e-9, T, F, want_final=True, table=tab[:, 1:])
    bad = tab.copy()
    bad[0, 7, 1] = np.nan
    with pytest.raises(_lib.SSSError, match="ENONFINITE"):
        plan.batch(flat, None, 0.0, 1e-9, T, F, want_final=True, table=bad)
    plan.set_batch_config(variant=1)
    with pytest.raises(_lib.SSSError, match="row-part"):
        plan.batch(flat, None, 0.0, 1e-9, T, F, want_final=True, table=tab)
    plan.set_batch_config(variant=0)
    _, fin = plan.batch(flat, None, 0.0, 1e-9, T, F, want_final=True, table=tab)
    # L0 alone (constant, folded): the free evolution from the same plan's programs
    prog = np.zeros((1, 4, 1, 5))
    prog[:, :, :, 0] = np.inf
    _, fin_p = plan.batch(flat, prog, 0.0, 1e-9, T, F, want_final=True)
    assert np.array_equal(fin, fin_p)
