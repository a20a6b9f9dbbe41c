"""Device-side health check of the batched kernels: every readout and
final-state value a kernel writes is tested, and the first NaN or infinity
turns the run's SSS_OK into SSS_ENONFINITE naming the trajectory and the
output sample.  The bad values come from host-made inputs (a readout that
overflows binary64, an infinite initial state); nothing faults."""
import numpy as np
import pytest

from conftest import load_case
from oracle import oracle

pytestmark = pytest.mark.gpu

# (lanes, variant) pairs that reach every batched kernel: lane groups,
# register rows, shuffles, row parts, slot-packed and phased row parts
KERNELS = [(4, 0), (16, 1), (8, 2), (32, 3), (32, 4), (128, 4), (16, 6), (128, 6), (32, 7)]


def _nv7_sweep(B=6):
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.quadratures import method
    c = load_case("nv7_n49")
    vm = c["vectorisation_map"]
    N = vm.shape[0]
    progs = np.zeros((B, 4, 1, 5))
    progs[:, :, :, 0] = np.inf
    progs[:, 0, 0, 2] = 5e6/28.025e9
    progs[:, 0, 0, 3] = 2.870e9 + 28.025e9*5e-3 + np.linspace(-30e6, 30e6, B)
    progs[:, 3, 0, 1] = 10/65.9
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    rho0 = np.stack([oracle.flatten(rho, vm, N)]*B)
    ground = [i for i, (y, x, ch) in enumerate(vm) if y == x == 1 and ch == 0]
    W, nodes = method(2)
    return _lib.Plan(c["generators"], W, nodes), rho0, progs, ground


@pytest.mark.parametrize("lanes,variant", KERNELS)
def test_overflowing_readout_is_reported(lanes, variant):
    """Trajectory 3 starts with its population scaled by 1e300 and the
    readout weighs that population by 1e10: its first readout overflows to
    infinity.  The run reports trajectory 3 at sample 0; the same plan's
    next run, on healthy inputs, returns normally."""
    from superspinsim_gb300 import _lib
    plan, rho0, progs, ground = _nv7_sweep()
    plan.set_batch_config(lanes=lanes, variant=variant)
    w = np.zeros(rho0.shape[1])
    w[ground] = 1e10
    bad = rho0.copy()
    bad[3] *= 1e300
    with pytest.raises(_lib.SSSError) as e:
        plan.batch(bad, progs, 0.0, 1e-9, 3, 20, readout_weights=w)
    assert e.value.code == -5
    assert "trajectory 3," in str(e.value) and "output sample 0" in str(e.value)
    ro, _ = plan.batch(rho0, progs, 0.0, 1e-9, 3, 20, readout_weights=w)
    assert np.isfinite(ro).all()


@pytest.mark.parametrize("lanes,variant", [(4, 0), (32, 4), (16, 6), (32, 7)])
def test_infinite_initial_state_is_reported_in_the_final_state(lanes, variant):
    """No readout: an infinite entry of trajectory 5's initial state turns
    its final state non-finite, which the final-state check catches."""
    from superspinsim_gb300 import _lib
    plan, rho0, progs, ground = _nv7_sweep()
    plan.set_batch_config(lanes=lanes, variant=variant)
    bad = rho0.copy()
    bad[5, ground] = np.inf
    with pytest.raises(_lib.SSSError) as e:
        plan.batch(bad, progs, 0.0, 1e-9, 2, 20, want_final=True)
    assert e.value.code == -5 and "trajectory 5," in str(e.value)


def test_chunked_launches_are_checked_after_the_run():
    """sss_batch_launch stays asynchronous; sss_batch_check reports the
    first bad value of the chunks and resets the word, so a second check
    passes."""
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.sweep import ChunkedRun, Sweep
    c = load_case("nv7_n49")
    _, rho0, progs, ground = _nv7_sweep(B=4)
    sweep = Sweep(c["generators"], c["vectorisation_map"], number_of_fine_divisions=20)
    w = np.zeros(rho0.shape[1])
    w[ground] = 1e10
    bad = rho0.copy()
    bad[2] *= 1e300
    run = ChunkedRun(sweep, bad, progs, 0.0, 1e-9, 4, readout_weights=w)
    run.step(2)
    run.step(2)
    with pytest.raises(_lib.SSSError) as e:
        run.results()
    assert e.value.code == -5 and "trajectory 2," in str(e.value)
    run.check()  # the word was reset
