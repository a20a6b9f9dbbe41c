"""The headline workload at its full size: 1024 NV-7 ODMR trajectories over
2 us at 5 ps (400,000 CF4:2 steps each).  Size-independent properties on
every trajectory, and one sampled trajectory against the oracle over the
whole run."""
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
    # one trajectory (the resonance neighbourhood: largest contrast) against
    # the oracle's vector mode over all 400,000 steps
    b = int(np.argmin(ro[:, -1]))
    W, nodes = quadrature(2)
    _, ref = oracle.simulate(gens, rho, 0.0, T*dt + 1e-13, dt, progs[b], K=2, W=W, nodes=nodes,
                             F=F, vectorisation_map=vm, mode="vector", degree=16, flat_out=True)
    assert np.abs(out["final"][b] - ref[-1]).max() <= 1e-10
    assert np.abs(ro[b] - ref @ w).max() <= 1e-9*np.abs(ref @ w).max()
    assert N == 49
