"""The batched kernels against the reference's own algorithm at full length.

The fixtures come from the oracle's reference mode (tests/golden/
make_golden.py fullrun): the reference's simulate restated loop for loop --
first-order Taylor after 4^-35 scaling, 70 residual squarings per
exponential, the serial chain of step propagators -- which reproduces the
reference's outputs bit for bit on every fixture it was checked against
(tests/test_oracle_golden.py).  They use the reference's own generators and
quadrature tables.

* NV-7 ODMR (49 x 49): the 1024-frequency sweep's trajectory nearest the
  ms=0 -> +1 line over all 400,000 steps (2 us at 5 ps): the fluorescence
  at every 1 ns sample and the full state every 100 ns.
* NV-21 (441 x 441): four trajectories of the 256-frequency sweep over
  104 steps of 5 ps, the full state at every output sample.

Bars: density max-abs <= 1e-10, fluorescence relative <= 1e-9."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_case, quadrature

pytestmark = pytest.mark.gpu

DENSITY_BAR, FLUOR_BAR = 1e-10, 1e-9


def _fixture(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("variant", [0, 4, 6])
def test_nv7_full_trajectory_matches_reference_algorithm(variant):
    from superspinsim_gb300 import _lib
    fx = _fixture("nv7_fullrun")
    c = load_case("nv7_n49")
    W, nodes = quadrature(2)
    T, dt, F = int(fx["T"]), float(fx["dt"]), int(fx["F"])
    plan = _lib.Plan(c["generators"], W, nodes)
    plan.set_batch_config(variant=variant)
    ro, fin, tr = plan.batch(fx["rho0"][None], fx["program"][None], 0.0, dt, T, F,
                             readout_weights=fx["readout_weights"], want_final=True,
                             want_trace=True)
    ref_f = fx["fluorescence"]
    assert np.abs(ro[0] - ref_f).max() <= FLUOR_BAR*np.abs(ref_f).max()
    assert np.abs(tr[0][fx["kept_samples"]] - fx["states"]).max() <= DENSITY_BAR
    assert np.abs(fin[0] - fx["states"][-1]).max() <= DENSITY_BAR


def test_nv7_sweep_row_matches_reference_algorithm():
    """The same trajectory inside the full 1024-frequency sweep (its row of
    the batch equals the run on its own)."""
    from superspinsim_gb300.sweep import Sweep
    fx = _fixture("nv7_fullrun")
    c = load_case("nv7_n49")
    vm = c["vectorisation_map"]
    T, dt, F = int(fx["T"]), float(fx["dt"]), int(fx["F"])
    progs = np.repeat(fx["program"][None], 1024, axis=0)
    progs[:, 0, 0, 3] = fx["freqs"]
    sw = Sweep(c["generators"], vm, number_of_exponentials=2, number_of_fine_divisions=F)
    out = sw.run(fx["rho0"][None], progs, 0.0, T*dt + 1e-13, dt,
                 readout_weights=fx["readout_weights"], final_state=True)
    b = int(fx["index"])
    ref_f = fx["fluorescence"]
    assert np.abs(out["readout"][b] - ref_f).max() <= FLUOR_BAR*np.abs(ref_f).max()
    assert np.abs(out["final"][b] - fx["states"][-1]).max() <= DENSITY_BAR


@pytest.mark.parametrize("lanes,variant", [(0, 0), (128, 4), (128, 6), (256, 6)])
def test_nv21_window_matches_reference_algorithm(lanes, variant):
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.sweep import population_weights
    fx = _fixture("nv21_window")
    c = load_case("nv21_n441")
    vm = c["vectorisation_map"]
    W, nodes = quadrature(2)
    T, dt, F = int(fx["T"]), float(fx["dt"]), int(fx["F"])
    plan = _lib.Plan(c["generators"], W, nodes)
    plan.set_batch_config(lanes=lanes, variant=variant)
    B = fx["programs"].shape[0]
    w = population_weights(vm, range(9, 18), 65.9e6)
    ro, fin, tr = plan.batch(np.repeat(fx["rho0"][None], B, axis=0), fx["programs"], 0.0, dt, T,
                             F, readout_weights=w, want_final=True, want_trace=True)
    ref = fx["states"]
    assert np.abs(tr - ref).max() <= DENSITY_BAR
    ref_f = ref @ w
    assert np.abs(ro - ref_f).max() <= FLUOR_BAR*np.abs(ref_f).max()
