"""Adjoint gradients (sss_adjoint_run) against central finite differences
of the GPU forward and of the CPU oracle."""
import numpy as np
import pytest

from conftest import load_case, quadrature
from oracle import oracle

pytestmark = pytest.mark.gpu

F_RES = 2.870e9 + 28.025e9*5e-3


def _problem(seed=5, B=3, S=4, seg=2e-9, t_read=4e-9):
    from superspinsim_gb300 import protocols
    rng = np.random.default_rng(seed)
    rabi = rng.uniform(5e6, 20e6, (B, S))
    phase = rng.uniform(0, 2*np.pi, (B, S))
    progs, dur = protocols.pulse_shapes(rabi, phase, seg, F_RES, 10/65.9, t_read)
    return rabi, phase, progs, dur


def _objective(name="nv7_n19"):
    from superspinsim_gb300.adjoint import Objective
    c = load_case(name)
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1
    return Objective(c["generators"], c["vectorisation_map"], rho, [3, 4, 5], 65.9e6,
                     number_of_fine_divisions=100), c, rho


@pytest.mark.parametrize("variant", [0, 4, 1])
def test_adjoint_objective_matches_forward_and_fd(variant):
    """variant 0: stored forward states and the slot-programmed backward
    (the block series on a phased or slot-packed program); variant 4: the
    same forward with the transposed row-part backward kernel; variant 1:
    the checkpointed adjoint kernel."""
    from superspinsim_gb300.adjoint import trapezoid_weights
    obj, c, rho = _objective()
    obj.plan.set_batch_config(variant=variant)
    rabi, phase, progs, dur = _problem()
    dt = 1e-9
    T = int(round(dur[0]/dt))
    S = rabi.shape[1]
    tw = trapezoid_weights(T, dt, int(round(S*2e-9/dt)) - 1, T - 1)
    J, grad = obj.run(progs, dt, T, tw)
    Jf = obj.forward_only(progs, dt, T, tw)
    # the adjoint's forward pass and forward_only may run different kernel
    # layouts (row parts with the usual Horner iterates, or the scaled
    # Horner of the phased and slot-packed kernels): equal to rounding
    assert np.abs(J - Jf).max() <= 1e-12*np.abs(Jf).max()
    # central differences of the GPU forward, all parameters in one batch,
    # Richardson-extrapolated from steps h and 2h (h = 1e-3): truncation
    # O(h^4) ~ 1e-12 and J's accumulated roundoff (~1e-14 relative) costs
    # ~1e-11 of J per unit derivative -- both far below the tolerance
    B = progs.shape[0]
    pert, idx = [], []
    for b in range(B):
        for s in range(S):
            for comp, col, h in ((0, 2, 1e-3*progs[b, 0, s, 2]), (1, 4, 1e-3)):
                for step in (h, -h, 2*h, -2*h):
                    p = progs[b].copy()
                    p[0, s, col] += step
                    pert.append(p)
                idx.append((b, s, comp, h))
    Jp = obj.forward_only(np.stack(pert), dt, T, tw)
    for k, (b, s, comp, h) in enumerate(idx):
        d1 = (Jp[4*k] - Jp[4*k + 1])/(2*h)
        d2 = (Jp[4*k + 2] - Jp[4*k + 3])/(4*h)
        fd = (4*d1 - d2)/3
        atol = 1e-11*abs(J[b])/h
        assert abs(grad[b, s, comp] - fd) <= 1e-7*abs(fd) + atol, (b, s, comp, grad[b, s, comp], fd)
    # and the plain central difference with h = 1e-6 (the workload's check)
    for k, (b, s, comp, h) in enumerate(idx[:4]):
        p1, p2 = progs[b].copy(), progs[b].copy()
        hh = h*1e-3
        col = 2 if comp == 0 else 4
        p1[0, s, col] += hh
        p2[0, s, col] -= hh
        Jc = obj.forward_only(np.stack([p1, p2]), dt, T, tw)
        fd = (Jc[0] - Jc[1])/(2*hh)
        assert abs(grad[b, s, comp] - fd) <= 1e-5*abs(fd) + 1e-13*abs(J[b])/hh


def _two_channel_problem():
    """Pulse shapes on x plus a y drive (half the amplitude, other phases,
    detuned by 2 MHz) on channel 1; the laser on channel 3 is off during
    the pulses and on for the readout."""
    rabi, phase, progs, dur = _problem(seed=11, B=2, S=3)
    progs[:, 1] = progs[:, 0]
    progs[:, 1, :3, 2] *= 0.5
    progs[:, 1, :3, 3] += 2e6
    progs[:, 1, :3, 4] += 0.7
    return progs, dur


@pytest.mark.parametrize("variant", [0, 4, 1])
@pytest.mark.parametrize("channel", [0, 1, 3])
def test_channel_adjoint_matches_fd(channel, variant):
    """sss_adjoint_run_channel: d J / d (amplitude, phase, offset, frequency)
    of the segments of the x drive, of a detuned y drive and of the laser,
    against Richardson-extrapolated central differences of the GPU forward.
    On channel 0 its first two entries equal sss_adjoint_run's bit for bit."""
    from superspinsim_gb300.adjoint import trapezoid_weights
    obj, c, rho = _objective()
    obj.plan.set_batch_config(variant=variant)
    progs, dur = _two_channel_problem()
    dt = 1e-9
    T = int(round(dur[0]/dt))
    tw = trapezoid_weights(T, dt, 5, T - 1)
    J, g4 = obj.run(progs, dt, T, tw, channel=channel)
    assert g4.shape == progs.shape[:1] + (progs.shape[2], 4)
    Jf = obj.forward_only(progs, dt, T, tw)
    assert np.abs(J - Jf).max() <= 1e-12*np.abs(Jf).max()
    if channel == 0:
        J2, g2 = obj.run(progs, dt, T, tw)
        assert np.array_equal(J2, J) and np.array_equal(g2, g4[..., :2])
    # (program column, step) per parameter: amplitude, phase, offset, frequency
    B, S = progs.shape[0], progs.shape[2]
    pert, idx = [], []
    for b in range(B):
        for s in range(S):
            seg = progs[b, channel, s]
            amp_h = 1e-3*max(abs(seg[2]), abs(seg[1]), 1e-3)
            for comp, col, h in ((0, 2, amp_h), (1, 4, 1e-3), (2, 1, amp_h), (3, 3, 1e4)):
                for step in (h, -h, 2*h, -2*h):
                    p = progs[b].copy()
                    p[channel, s, col] += step
                    pert.append(p)
                idx.append((b, s, comp, h))
    Jp = obj.forward_only(np.stack(pert), dt, T, tw)
    scale = np.abs(g4).max()
    for k, (b, s, comp, h) in enumerate(idx):
        d1 = (Jp[4*k] - Jp[4*k + 1])/(2*h)
        d2 = (Jp[4*k + 2] - Jp[4*k + 3])/(4*h)
        fd = (4*d1 - d2)/3
        atol = 1e-11*abs(J[b])/h + 1e-9*scale
        assert abs(g4[b, s, comp] - fd) <= 1e-6*abs(fd) + atol, \
            (b, s, comp, g4[b, s, comp], fd)
    if channel == 3:
        # a constant segment: d/d amplitude = d/d offset, phase and frequency 0
        assert np.array_equal(g4[..., 0], g4[..., 2])
        assert not g4[..., 1].any() and not g4[..., 3].any()


@pytest.mark.parametrize("n_shapes", [3, 600])
def test_slot_backward_equals_row_part_backward(n_shapes):
    """The slot-programmed backward (the block series on a slot program; 64
    lanes for the small batch, 32 for the large one) and the row-part
    backward evaluate the same truncated series in different orders: equal
    objectives and gradients to rounding, on the x drive and on the laser."""
    from superspinsim_gb300.adjoint import trapezoid_weights
    obj, c, rho = _objective()
    rabi, phase, progs, dur = _problem(seed=13, B=3, S=3)
    progs = progs[np.arange(n_shapes) % 3]
    dt = 1e-9
    T = int(round(dur[0]/dt))
    tw = trapezoid_weights(T, dt, 5, T - 1)
    out = {}
    for variant in (0, 4):
        obj.plan.set_batch_config(variant=variant)
        out[variant] = (obj.run(progs, dt, T, tw), obj.run(progs, dt, T, tw, channel=3),
                        obj.plan.batch_info())
    assert out[0][2]["variant"] in (6, 7) and out[4][2]["variant"] == 4
    assert out[0][2]["lanes"] == (64 if n_shapes == 3 else 32)
    for k in range(2):
        (J0, g0), (J4, g4) = out[0][k], out[4][k]
        assert np.abs(J0 - J4).max() <= 1e-13*np.abs(J4).max()
        assert np.abs(g0 - g4).max() <= 1e-10*np.abs(g4).max()


def test_channel_adjoint_rejects_a_channel_without_generator():
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.adjoint import trapezoid_weights
    obj, c, rho = _objective()
    progs, dur = _two_channel_problem()
    T = int(round(dur[0]/1e-9))
    tw = trapezoid_weights(T, 1e-9, 5, T - 1)
    with pytest.raises(_lib.SSSError) as e:
        obj.run(progs, 1e-9, T, tw, channel=4)
    assert e.value.code == -1


def test_adjoint_matches_fd_of_oracle():
    """Finite differences of the CPU oracle in reference mode (the
    reference's own algorithm: 4^-35 scaling and 70 residual squarings per
    exponential) on one shape with two segments."""
    from superspinsim_gb300.adjoint import trapezoid_weights
    obj, c, rho = _objective()
    rabi, phase, progs, dur = _problem(seed=9, B=1, S=2, seg=1e-9, t_read=2e-9)
    dt = 1e-9
    T = int(round(dur[0]/dt))
    tw = trapezoid_weights(T, dt, 1, T - 1)
    J, grad = obj.run(progs, dt, T, tw)
    W, nodes = quadrature(2)
    vm = c["vectorisation_map"]

    def J_oracle(p):
        _, d = oracle.simulate(c["generators"], rho, 0.0, T*dt + 1e-13, dt, p, K=2, W=W,
                               nodes=nodes, F=100, vectorisation_map=vm, mode="reference",
                               flat_out=True)
        return float((d @ obj.rw) @ tw)

    assert abs(J_oracle(progs[0]) - J[0]) <= 1e-11*abs(J[0])
    for s in range(2):
        for comp, col, h in ((0, 2, 1e-6*progs[0, 0, s, 2]), (1, 4, 1e-6)):
            pp, pm = progs[0].copy(), progs[0].copy()
            pp[0, s, col] += h
            pm[0, s, col] -= h
            fd = (J_oracle(pp) - J_oracle(pm))/(2*h)
            assert abs(grad[0, s, comp] - fd) <= 1e-5*abs(fd) + 1e-9*abs(J[0]), (s, comp)


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    from superspinsim_gb300.adjoint import make_pulse_function
    obj, c, rho = _objective()
    fn = make_pulse_function(obj, 2e-9, F_RES, 10/65.9, 4e-9, 1e-9)
    rabi, phase, progs, dur = _problem(B=2, S=3)
    r = torch.tensor(rabi, requires_grad=True)
    p = torch.tensor(phase, requires_grad=True)
    J = fn.apply(r, p)
    J.sum().backward()
    assert r.grad.shape == r.shape and p.grad.shape == p.shape
    # one directional derivative against a forward difference pair
    with torch.no_grad():
        h = 1e-6
        d = torch.zeros_like(p)
        d[0, 1] = h
        fd = (fn.apply(r, p + d) - fn.apply(r, p - d))[0]/(2*h)
    assert abs(float(p.grad[0, 1]) - float(fd)) <= 1e-5*abs(float(fd)) + 1e-12


def test_adjoint_chunks_and_memory_fallback():
    """Stored-state memory bounded to one trajectory: chunked runs give the
    same J and gradients bit for bit; bounded below one trajectory: the
    checkpointed adjoint runs instead and agrees to rounding."""
    from superspinsim_gb300.adjoint import trapezoid_weights
    obj, c, rho = _objective()
    rabi, phase, progs, dur = _problem(seed=13, B=5, S=3)
    dt = 1e-9
    T = int(round(dur[0]/dt))
    tw = trapezoid_weights(T, dt, int(round(3*2e-9/dt)) - 1, T - 1)
    J, grad = obj.run(progs, dt, T, tw)
    info = obj.plan.batch_info()
    per_traj = T*obj.F*2*info["rows"]*8
    obj.plan.set_adjoint_memory(per_traj + 8)
    J1, g1 = obj.run(progs, dt, T, tw)
    assert obj.plan.last_launches() == 2*progs.shape[0]
    assert np.array_equal(J1, J) and np.array_equal(g1, grad)
    obj.plan.set_adjoint_memory(per_traj // 2)
    J2, g2 = obj.run(progs, dt, T, tw)
    assert obj.plan.last_launches() == 1
    assert np.abs(J2 - J).max() <= 1e-12*np.abs(J).max()
    assert np.abs(g2 - grad).max() <= 1e-9*np.abs(grad).max()


def test_adjoint_nv21_wide_groups_match_fd():
    """21-level NV with 14N (441 x 441): the row-part adjoint with groups
    wider than a warp (one trajectory per CTA), J against the forward and
    the gradient against Richardson-extrapolated central differences."""
    from superspinsim_gb300 import protocols
    from superspinsim_gb300.adjoint import Objective, trapezoid_weights
    c = load_case("nv21_n441")
    rho = np.zeros((21, 21), complex)
    for k in range(3, 6):
        rho[k, k] = 1/3
    obj = Objective(c["generators"], c["vectorisation_map"], rho, list(range(9, 18)), 65.9e6,
                    number_of_fine_divisions=50)
    rng = np.random.default_rng(17)
    B, S = 2, 2
    rabi = rng.uniform(5e6, 20e6, (B, S))
    phase = rng.uniform(0, 2*np.pi, (B, S))
    f_c = 2.870e9 + 28.025e9*0.05
    progs, dur = protocols.pulse_shapes(rabi, phase, 1e-9, f_c, 10/65.9, 2e-9)
    dt = 1e-9
    T = int(round(dur[0]/dt))
    tw = trapezoid_weights(T, dt, S - 1, T - 1)
    J, grad = obj.run(progs, dt, T, tw)
    assert obj.plan.last_launches() == 2     # row-part forward + backward, no fallback
    assert obj.plan.batch_info()["lanes"] > 32
    Jf = obj.forward_only(progs, dt, T, tw)
    # the adjoint's forward pass and forward_only may run different kernel
    # layouts (row parts with the usual Horner iterates, or the scaled
    # Horner of the phased and slot-packed kernels): equal to rounding
    assert np.abs(J - Jf).max() <= 1e-12*np.abs(Jf).max()
    pert, idx = [], []
    for b in range(B):
        for s in range(S):
            for comp, col, h in ((0, 2, 1e-3*progs[b, 0, s, 2]), (1, 4, 1e-3)):
                for step in (h, -h, 2*h, -2*h):
                    p = progs[b].copy()
                    p[0, s, col] += step
                    pert.append(p)
                idx.append((b, s, comp, h))
    Jp = obj.forward_only(np.stack(pert), dt, T, tw)
    for k, (b, s, comp, h) in enumerate(idx):
        d1 = (Jp[4*k] - Jp[4*k + 1])/(2*h)
        d2 = (Jp[4*k + 2] - Jp[4*k + 3])/(4*h)
        fd = (4*d1 - d2)/3
        assert abs(grad[b, s, comp] - fd) <= 1e-7*abs(fd) + 1e-11*abs(J[b])/h, (b, s, comp)
