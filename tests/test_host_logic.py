"""Host-side logic of the package, without a GPU: sample counting, the
flattened state layouts, the sampler-table row order, coefficient programs
and the protocol and readout builders."""
import math

import numpy as np
import pytest

from conftest import load_case
from oracle import oracle


def test_number_of_samples_truncates_like_the_reference():
    # superspinsim/generate_simulator.py:1519: int((tf - t0)/dt)
    from superspinsim_gb300.generate_simulator import number_of_samples
    assert number_of_samples(0.0, 100e-9, 1e-9) == 99
    assert number_of_samples(0.0, 100e-9 + 1e-13, 1e-9) == 100
    assert number_of_samples(0.0, 0.5e-9, 1e-9) == 0
    for t0, tf, dt in ((0.0, 10e-6, 1e-9), (1e-9, 7e-9, 2e-9), (0.0, 2e-6, 1e-9)):
        assert number_of_samples(t0, tf, dt) == oracle.number_of_samples(t0, tf, dt)


@pytest.mark.parametrize("hermitian", [True, False])
def test_flatten_unflatten_round_trip(hermitian):
    """The Hermitian basis (vectorisation-map rows y, x, re/im, the lower
    triangle mirrored) and the complex basis (all n^2 entries, re/im
    interleaved, row-major) against the oracle's flattening."""
    from superspinsim_gb300.generate_simulator import flatten_density, unflatten_density
    c = load_case("nv7_n49")
    vm = c["vectorisation_map"] if hermitian else None
    N = 49 if hermitian else 98
    rng = np.random.default_rng(2)
    a = rng.normal(size=(3, 7, 7)) + 1j*rng.normal(size=(3, 7, 7))
    h = a + np.conj(np.swapaxes(a, 1, 2)) if hermitian else a
    flat = flatten_density(h, N, vm)
    assert flat.shape == (3, N)
    for b in range(3):
        assert np.array_equal(flat[b], oracle.flatten(h[b], vm, N))
    back = unflatten_density(flat, 7, vm)
    assert np.array_equal(back, h)


def test_sample_table_row_order():
    """Row (r*T + t)*Q + k of a sampled table is the sampler's row at node
    k of fine step r of output sample t, at the reference's node time
    ((t0 + (r*dt)/F) + dt*t) + (dt*node)/F, the row zeroed first."""
    from superspinsim_gb300.generate_simulator import sample_table
    nodes = np.array([0.2113248654051871, 0.7886751345948129])
    t0, dt, T, F, G = 3e-9, 1e-9, 4, 5, 3
    seen = []

    def sampler(time, row):
        assert np.all(row == 0.0)
        row[0] = time
        row[2] = 1.0
        seen.append(time)

    tab = sample_table(sampler, G, t0, dt, T, F, nodes)
    assert tab.shape == (1, F*T*len(nodes), G)
    for r in range(F):
        for t in range(T):
            for k in range(len(nodes)):
                tn = ((t0 + (r*dt)/F) + dt*t) + (dt*nodes[k])/F
                assert tab[0, (r*T + t)*len(nodes) + k, 0] == tn
    assert np.all(tab[0, :, 1] == 0.0) and np.all(tab[0, :, 2] == 1.0)
    assert len(seen) == F*T*len(nodes)


def test_program_segments_and_arrays():
    """First segment with t < t_end gives offset + amplitude*cos(tau f t +
    phase); after the last, 0.  as_array pads unused segments with
    t_end = -inf (never match); stack pads shorter programs the same way."""
    from superspinsim_gb300.program import Program, array_value, stack
    p = Program().add("x", 2e-9, offset=0.5).add("x", 5e-9, amplitude=2.0, frequency=1e8,
                                                  phase=0.3)
    p.add("r", np.inf, offset=0.25)
    assert p.value(0, 1e-9) == 0.5
    assert p.value(0, 3e-9) == 2.0*math.cos(math.tau*1e8*3e-9 + 0.3)
    assert p.value(0, 5e-9) == 0.0
    assert p.value(3, 1.0) == 0.25 and p.value(1, 1e-9) == 0.0
    a = p.as_array()
    assert a.shape == (4, 2, 5) and a[1, 0, 0] == -np.inf and a[3, 1, 0] == -np.inf
    for ch in range(4):
        for t in (0.0, 1e-9, 2e-9, 3e-9, 4.99e-9, 6e-9):
            assert array_value(a, ch, t) == p.value(ch, t)
    s = stack([p, Program().add("z", 1e-9, offset=1.0)])
    assert s.shape == (2, 4, 2, 5) and s[1, 2, 1, 0] == -np.inf
    assert p.bound() == [2.0, 0.0, 0.0, 0.25]
    with pytest.raises(ValueError):
        p.as_array(nseg=1)


def test_protocol_builders():
    """ODMR, Ramsey and pulse-shape programs: segment boundaries and
    durations as their docstrings state."""
    from superspinsim_gb300 import protocols
    from superspinsim_gb300.program import array_value
    g = protocols.GAMMA
    o = protocols.odmr([1e9, 2e9], 5e6, 0.1)
    assert o.shape == (2, 4, 1, 5)
    assert array_value(o[1], 0, 1e-6) == (5e6/g)*math.cos(math.tau*2e9*1e-6)
    assert array_value(o[0], 3, 7.0) == 0.1
    rabi, det, tau = np.array([4e6]), np.array([1e6]), np.array([2e-7])
    p, dur = protocols.ramsey(rabi, det, tau, 3e9, 0.2, t_init=1e-6, t_read=5e-7)
    tp = 1/(4*4e6)
    assert dur[0] == pytest.approx(1e-6 + 2*tp + 2e-7 + 5e-7, rel=1e-15)
    assert array_value(p[0], 3, 0.5e-6) == 0.2          # laser on while initialising
    assert array_value(p[0], 3, 1e-6 + tp/2) == 0.0     # off during the pulses and tau
    assert array_value(p[0], 0, 1e-6 + tp + 1e-7) == 0.0   # free precession
    t_mid = 1e-6 + tp/2
    assert array_value(p[0], 0, t_mid) == (4e6/g)*math.cos(math.tau*(3e9 + 1e6)*t_mid)
    assert array_value(p[0], 3, dur[0] - 1e-9) == 0.2   # readout
    amps, phs = np.array([[1e6, 2e6, 3e6]]), np.array([[0.0, 1.0, 2.0]])
    q, d2 = protocols.pulse_shapes(amps, phs, 2e-9, 3e9, 0.3, 1e-8)
    assert q.shape == (1, 4, 4, 5) and d2[0] == pytest.approx(6e-9 + 1e-8, rel=1e-15)
    assert array_value(q[0], 0, 3e-9) == (2e6/g)*math.cos(math.tau*3e9*3e-9 + 1.0)
    assert array_value(q[0], 0, 7e-9) == 0.0 and array_value(q[0], 3, 7e-9) == 0.3
    assert array_value(q[0], 3, 5e-9) == 0.0


def test_readout_and_time_weights():
    from superspinsim_gb300.adjoint import trapezoid_weights
    from superspinsim_gb300.sweep import population_weights, trapezoid
    c = load_case("nv7_n49")
    vm = c["vectorisation_map"]
    w = population_weights(vm, [3, 4, 5], scale=2.0)
    rho = np.diag(np.arange(1.0, 8.0)).astype(complex)
    assert w @ oracle.flatten(rho, vm, 49) == 2.0*(4 + 5 + 6)
    tw = trapezoid_weights(10, 1e-9, 2, 8)
    assert tw.sum() == pytest.approx(6e-9, rel=1e-15)
    assert tw[2] == tw[8] == 0.5e-9 and tw[1] == 0.0 and tw[9] == 0.0
    r = np.array([[1.0, 2.0, 3.0]])
    assert trapezoid(r, 1e-9, initial=0.0)[0] == pytest.approx(1e-9*(0.5*0 + 1 + 2 + 0.5*3))
