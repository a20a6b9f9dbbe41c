"""Equivalence-class (kernel) and unitary modes of the plain path, through
the C-ABI: against their oracle restatements, against the Liouvillian path
on the same system, and against the reference's own qutrit output."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, load_case, quadrature
from oracle import oracle

pytestmark = pytest.mark.gpu

sys.path.insert(0, GOLDEN)
import make_golden as mg  # noqa: E402  (case definitions only)

T_DRIVE = mg.drive(7e6, 10e-6)          # x field of the qutrit cases (tesla)


def _program(x_segs, y_segs=None):
    return mg.program_array([x_segs, y_segs or mg.ZERO, mg.ZERO, mg.ZERO])


def _modes(name):
    with np.load(os.path.join(GOLDEN, f"modes_{name}.npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("K", [1, 2])
def test_kernel_mode_matches_oracle_and_full_space(K):
    """The reference's projection (its find_kernel output for the qutrit):
    the lifted result equals the oracle's restatement and the unprojected
    run, the identity direction being stationary."""
    from superspinsim_gb300 import generate_simulator
    z = _modes("qutrit")
    vm, P, gi = z["vectorisation_map"], z["image_projection"], z["generators_image"]
    # lab-frame sampler rows [1, x, y, z, r]; the projected generators keep
    # that order
    prog = _program(T_DRIVE)
    rho = np.diag([0.2, 0.3, 0.5]).astype(complex)
    rho[0, 2] = rho[2, 0] = 0.1
    W, nodes = quadrature(K)
    sim_k = generate_simulator(prog, gi, vm, number_of_exponentials=K,
                               number_of_fine_divisions=50, use_kernel=True,
                               image_projection=P, full_projection=z["full_projection"])
    t, dk = sim_k(rho, 0.0, 5e-9 + 1e-13, 1e-9)
    sim_f = generate_simulator(prog, z["generators"], vm, number_of_exponentials=K,
                               number_of_fine_divisions=50)
    _, df = sim_f(rho, 0.0, 5e-9 + 1e-13, 1e-9)
    _, do = oracle.simulate_kernel(gi, P, rho, 0.0, 5e-9 + 1e-13, 1e-9, prog,
                                   vectorisation_map=vm, K=K, W=W, nodes=nodes, F=50,
                                   mode="vector", degree=16)
    assert dk.shape == (5, 3, 3)
    assert np.abs(dk - do).max() <= 1e-12
    assert np.abs(dk - df).max() <= 1e-12
    # traces stay 1 and the state stays Hermitian
    assert np.abs(np.trace(dk, axis1=1, axis2=2) - 1).max() <= 1e-12
    assert np.abs(dk - np.conj(np.transpose(dk, (0, 2, 1)))).max() == 0.0


@pytest.mark.parametrize("drive_axis", ["x", "y"])
@pytest.mark.parametrize("rot", [False, True])
def test_unitary_mode_matches_oracle(drive_axis, rot):
    """The reference's operator generators; the device's conj(U) rho0 U^T
    against the oracle's column-by-column propagation, lab and rotating
    frame, x and y drives."""
    from superspinsim_gb300 import generate_simulator
    from superspinsim_gb300.rotating import make_rotating
    z = _modes("qutrit")
    vm = z["vectorisation_map"]
    gens = np.array([z["unitary_" + k] for k in ("H0", "Gx", "Gy", "Gz", "Gr")])
    prog = _program(T_DRIVE) if drive_axis == "x" else _program(mg.ZERO, T_DRIVE)
    rho = np.diag([0.1, 0.3, 0.6]).astype(complex)
    rho[0, 1], rho[1, 0] = 0.05 + 0.02j, 0.05 - 0.02j
    W, nodes = quadrature(2)
    kw = dict(number_of_exponentials=2, number_of_fine_divisions=50, use_unitary=True,
              elimination=z["elimination"], duplication=z["duplication"])
    rot_args, orot = {}, None
    g_in = gens
    if rot:
        new, V, Vi, d, s = make_rotating(gens[0], list(gens[1:]))
        rot_args = dict(use_rotating=True, vectors_real=V, inv_vectors_real=Vi, doubles=d,
                        singles=s)
        orot = dict(generators_rotating=np.array(new), vectors_real=V, inv_vectors_real=Vi,
                    doubles=np.asarray(d).reshape(-1, 2), singles=s)
        g_in = np.array(new)   # rotating rows are [x, y, z, r]: the same channels
    sim = generate_simulator(prog, g_in, vm, **kw, **rot_args)
    _, du = sim(rho, 0.0, 5e-9 + 1e-13, 1e-9)
    _, do = oracle.simulate_unitary(gens, rho, 0.0, 5e-9 + 1e-13, 1e-9, prog,
                                    vectorisation_map=vm, rotating=orot, K=2, W=W,
                                    nodes=nodes, F=50, mode="vector", degree=16)
    assert np.abs(du - do).max() <= 1e-12


@pytest.mark.parametrize("rot", [False, True])
def test_unitary_and_kernel_front_ends_match_liouvillian(rot):
    """simspins on the qutrit with an x drive: the unitary and the
    equivalence-class modes give the Liouvillian mode's densities."""
    from superspinsim_gb300.sugar import simspins
    fns = [mg.channel_fn(s) for s in (T_DRIVE, mg.ZERO, mg.ZERO, mg.ZERO)]
    rho = np.diag([0.0, 0.0, 1.0]).astype(complex)
    args = (fns, 0.0, 5e-9, 1e-9, mg.QUTRIT, [{}], {}, rho)
    kw = dict(number_of_exponentials=5, number_of_fine_divisions=100, use_rotating=rot)
    _, dl = simspins(*args, **kw)
    _, du = simspins(*args, use_unitary=True, **kw)
    _, dk = simspins(*args, use_kernel=True, **kw)
    assert np.abs(du - dl).max() <= 1e-11
    assert np.abs(dk - dl).max() <= 1e-11


def test_unitary_front_end_matches_reference_output():
    """The reference's qutrit-couple run (Liouvillian, residual, CF2:1,
    F = 100) against simspins in unitary mode."""
    from superspinsim_gb300.sugar import simspins
    ref = load_case("qutrit_couple")
    fns = [mg.channel_fn(s) for s in (T_DRIVE, mg.ZERO, mg.ZERO, mg.ZERO)]
    _, du = simspins(fns, 0.0, 5e-9, 1e-9, mg.QUTRIT, [{}], {}, ref["rho0"],
                     number_of_exponentials=1, number_of_fine_divisions=100,
                     use_rotating=False, use_unitary=True)
    assert np.abs(du - ref["density"]).max() <= 1e-11


def test_modes_reject_batched_runs():
    from superspinsim_gb300 import _lib
    z = _modes("qutrit")
    W, nodes = quadrature(2)
    plan = _lib.Plan(np.array([z["unitary_" + k] for k in ("H0", "Gx", "Gy", "Gz", "Gr")]),
                     W, nodes)
    plan.set_unitary(3, z["vectorisation_map"])
    progs = _program(T_DRIVE)[None]
    with pytest.raises(_lib.SSSError, match="unitary"):
        plan.batch(np.zeros((1, 6)), progs, 0.0, 1e-9, 2, 10, want_final=True)
    with pytest.raises(_lib.SSSError):
        plan.set_projection(np.eye(6))
