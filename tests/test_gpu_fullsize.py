"""Every benchmark workload at its full size -- the spin-1 and NV-7 ODMR
sweeps, the 4096-trajectory Ramsey batch, the NV-21 sweep and the two
adjoint workloads: size-independent properties on every trajectory (density
matrices, zero padding, batch independence, objective consistency) and
sampled trajectories against the oracle or against finite differences."""
import numpy as np
import pytest

from conftest import quadrature
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_odmr_full_size_properties_and_sampled_parity():
    import bench
    from superspinsim_gb300.generate_simulator import unflatten_density
    from superspinsim_gb300.sweep import Sweep, population_weights
    gens, vm = bench.nv7_model()
    progs, rho = bench.workload(1024)
    N = vm.shape[0]
    dt, F, T = bench.DT_OUT, bench.F, int(round(bench.DURATION/bench.DT_OUT))
    sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F)
    w = population_weights(vm, [3, 4, 5])
    out = sw.run(rho, progs, 0.0, T*dt + 1e-13, dt, readout_weights=w, final_state=True)
    fin = unflatten_density(out["final"], 7, vm)
    # trace 1, Hermitian, populations in [0, 1], positive semidefinite
    assert np.abs(np.trace(fin, axis1=1, axis2=2) - 1).max() <= 1e-12
    pops = np.real(np.diagonal(fin, axis1=1, axis2=2))
    assert pops.min() >= -1e-12 and pops.max() <= 1 + 1e-12
    assert np.linalg.eigvalsh(fin).min() >= -1e-12
    ro = out["readout"]
    assert ro.shape == (1024, T) and np.all(np.isfinite(ro))
    # the trajectory nearest the ms=0 -> +1 line against the reference's own
    # algorithm (70 squarings per exponential) over all 400,000 steps: the
    # fixture made by the oracle's reference mode (tests/golden/make_golden.py
    # fullrun)
    import os
    from conftest import GOLDEN
    with np.load(os.path.join(GOLDEN, "nv7_fullrun.npz")) as z:
        b, ref_f, ref_fin = int(z["index"]), z["fluorescence"], z["states"][-1]
        assert np.array_equal(z["program"], progs[b])
    assert np.abs(out["final"][b] - ref_fin).max() <= 1e-10
    assert np.abs(65.9e6*ro[b] - ref_f).max() <= 1e-9*np.abs(ref_f).max()
    assert N == 49


def _check_densities(fin, n, vm, tol=1e-12):
    """Trace 1, populations in [0, 1] and positive semidefinite."""
    from superspinsim_gb300.generate_simulator import unflatten_density
    d = unflatten_density(fin, n, vm)
    assert np.abs(np.trace(d, axis1=1, axis2=2) - 1).max() <= tol
    pops = np.real(np.diagonal(d, axis1=1, axis2=2))
    assert pops.min() >= -tol and pops.max() <= 1 + tol
    assert np.linalg.eigvalsh(d).min() >= -tol


def test_spin1_full_sweep_against_oracle():
    """The spin-1 ODMR sweep at its full size (64 frequencies over +-20 MHz,
    200 ns at 10 ps, ms=0 population every 1 ns): every trajectory of the
    batched path against the oracle's vector mode, a quarter of them against
    the reference's algorithm (70 squarings per exponential), and the plain
    drop-in (the reference's exponential) on two of them."""
    from conftest import load_case
    from superspinsim_gb300 import generate_simulator
    from superspinsim_gb300.generate_simulator import unflatten_density
    from superspinsim_gb300.sweep import Sweep, population_weights
    c = load_case("spin1_c1")
    gens, vm, rho = c["generators"], c["vectorisation_map"], c["rho0"]
    f_res = 2.870e9 + 28.025e9*0.01
    progs = np.repeat(c["program"][None], 64, axis=0)
    progs[:, 0, 0, 3] = f_res + np.linspace(-20e6, 20e6, 64)
    T, dt, F = 200, 1e-9, 100
    W, nodes = quadrature(2)
    w = population_weights(vm, [1])
    sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F)
    out = sw.run(rho, progs, 0.0, T*dt + 1e-13, dt, readout_weights=w, final_state=True)
    _check_densities(out["final"], 3, vm)
    rhos = np.stack([rho]*64)
    _, refv = oracle.simulate(gens, rhos, 0.0, T*dt + 1e-13, dt, progs, K=2, W=W, nodes=nodes,
                              F=F, vectorisation_map=vm, mode="vector", degree=16,
                              flat_out=True)
    assert np.abs(out["final"] - refv[:, -1]).max() <= 1e-12
    assert np.abs(out["readout"] - refv @ w).max() <= 1e-12
    sub = np.arange(0, 64, 4)
    _, refr = oracle.simulate(gens, rhos[sub], 0.0, T*dt + 1e-13, dt, progs[sub], K=2, W=W,
                              nodes=nodes, F=F, vectorisation_map=vm, flat_out=True)
    assert np.abs(out["final"][sub] - refr[:, -1]).max() <= 1e-10
    rel = np.abs(out["readout"][sub] - refr @ w).max()/np.abs(refr @ w).max()
    assert rel <= 1e-9
    for i in (3, 8):
        sim = generate_simulator(progs[sub[i]], gens, vm, number_of_exponentials=2,
                                 number_of_fine_divisions=F, expm="reference")
        _, d = sim(rho, 0.0, T*dt + 1e-13, dt)
        assert d.shape == (T, 3, 3)
        assert np.abs(d - unflatten_density(refr[i], 3, vm)).max() <= 1e-12


def test_ramsey_full_size_properties_and_sampled_parity():
    """The batched Ramsey workload at full size (4096 seeded trajectories of
    uneven length, about 3.3e9 steps in one persistent launch): every final
    state a density matrix, readout rows zero after each trajectory's last
    sample, the eight shortest trajectories run as a batch of their own
    equal to their rows of the full batch (order and batch composition do
    not change a trajectory), and the shortest against the oracle over its
    whole length."""
    import argparse
    import bench
    from superspinsim_gb300.sweep import Sweep, population_weights
    args = argparse.Namespace(n_traj=0, duration=bench.DURATION)
    gens, vm, progs, rho, samples, T, levels, _ = bench.build_workload("ramsey", args)
    assert progs.shape[0] == 4096
    dt, F = bench.DT_OUT, bench.F
    w = population_weights(vm, levels)
    sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F)
    out = sw.run(rho, progs, 0.0, T*dt + 1e-13, dt, samples=samples, readout_weights=w,
                 final_state=True)
    ro = out["readout"]
    # up to 1.5 million steps: the generators' column sums are zero only to
    # rounding (about 1e-17 of the trace per step), so the trace may drift
    # by a few 1e-12 over the longest trajectories
    _check_densities(out["final"], 7, vm, tol=1e-11)
    assert np.all(np.isfinite(ro)) and ro.min() >= -1e-12 and ro.max() <= 1 + 1e-12
    pad = np.arange(T)[None, :] >= samples[:, None]
    assert np.all(ro[pad] == 0.0)
    short = np.argsort(samples, kind="stable")[:8]
    alone = sw.run(rho, progs[short], 0.0, T*dt + 1e-13, dt, samples=samples[short],
                   readout_weights=w, final_state=True)
    assert np.abs(alone["final"] - out["final"][short]).max() <= 1e-12
    assert np.abs(alone["readout"] - ro[short]).max() <= 1e-12
    b = int(short[0])
    n = int(samples[b])
    W, nodes = quadrature(2)
    _, ref = oracle.simulate(gens, rho, 0.0, n*dt + 1e-13, dt, progs[b], K=2, W=W, nodes=nodes,
                             F=F, vectorisation_map=vm, mode="vector", degree=16, flat_out=True)
    assert np.abs(out["final"][b] - ref[-1]).max() <= 1e-10
    assert np.abs(ro[b, :n] - ref @ w).max() <= 1e-9*np.abs(ref @ w).max()


def test_nv21_full_size_properties_and_window_parity():
    """The NV-21 (14N) sweep at full size (256 frequencies x 1 us at 5 ps,
    Liouvillian 441 x 441): every final state a density matrix, and the
    first five output samples (1,000 steps) of the trajectory nearest
    resonance against the oracle's dense vector mode."""
    import argparse
    import bench
    from superspinsim_gb300.sweep import Sweep, population_weights
    args = argparse.Namespace(n_traj=0, duration=bench.DURATION)
    gens, vm, progs, rho, _, T, levels, _ = bench.build_workload("nv21", args)
    assert progs.shape[0] == 256 and T == 1000 and vm.shape[0] == 441
    dt, F = bench.DT_OUT, bench.F
    w = population_weights(vm, levels)
    sw = Sweep(gens, vm, number_of_exponentials=2, number_of_fine_divisions=F)
    out = sw.run(rho, progs, 0.0, T*dt + 1e-13, dt, readout_weights=w, final_state=True)
    _check_densities(out["final"], 21, vm)
    ro = out["readout"]
    assert np.all(np.isfinite(ro))
    b = int(np.argmin(ro[:, -1]))
    W, nodes = quadrature(2)
    n = 5
    _, ref = oracle.simulate(gens, rho, 0.0, n*dt + 1e-13, dt, progs[b], K=2, W=W, nodes=nodes,
                             F=F, vectorisation_map=vm, mode="vector", degree=16, flat_out=True)
    assert np.abs(ro[b, :n] - ref @ w).max() <= 1e-12*np.abs(ref @ w).max()


@pytest.mark.parametrize("nv21", [False, True], ids=["nv7", "nv21"])
def test_adjoint_full_size_against_fd(nv21):
    """The adjoint workloads at full size (NV-7: 256 shapes x 128 segments,
    111,200 steps each; NV-21: 32 shapes x 64 segments): objectives equal to
    the forward kernel's, all gradients finite, and four gradient entries of
    one shape against central differences of the GPU forward with h = 1e-6
    (relative for amplitudes)."""
    import bench
    obj, progs, T, tw, S, _ = bench.adjoint_workload(nv21)
    dt = bench.DT_OUT
    J, grad = obj.run(progs, dt, T, tw)
    B = progs.shape[0]
    # S pulse segments and the readout segment of channel 0
    assert grad.shape == (B, S + 1, 2) and np.all(np.isfinite(grad)) and np.all(J > 0)
    Jf = obj.forward_only(progs, dt, T, tw)
    # the adjoint's forward pass and forward_only may run different kernel
    # layouts (row parts with the usual Horner iterates, or the scaled
    # Horner of the phased and slot-packed kernels): equal to rounding
    assert np.abs(J - Jf).max() <= 1e-12*np.abs(Jf).max()
    b = 1
    pert, idx = [], []
    for s in (0, S//2, S - 1):
        for comp, col in ((0, 2), (1, 4)):
            h = 1e-6*progs[b, 0, s, 2] if comp == 0 else 1e-6
            if h == 0.0:
                continue
            for step in (h, -h):
                p = progs[b].copy()
                p[0, s, col] += step
                pert.append(p)
            idx.append((s, comp, h))
    Jp = obj.forward_only(np.stack(pert), dt, T, tw)
    for k, (s, comp, h) in enumerate(idx):
        fd = (Jp[2*k] - Jp[2*k + 1])/(2*h)
        assert abs(grad[b, s, comp] - fd) <= 1e-5*abs(fd) + 1e-13*abs(J[b])/h, \
            (s, comp, grad[b, s, comp], fd)
