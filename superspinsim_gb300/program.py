"""Coefficient programs: time-dependent control amplitudes evaluated on the
GPU.

The reference's extension point is a numba-compiled sampler
``sampler(time, row)`` that writes the generator coefficients at a time
(superspinsim/generate_simulator.py:235-271; the front end builds it from
four Python callables -- x, y, z field in tesla and optical excitation --
in superspinsim/generate_generators.py:2317-2358).  Arbitrary Python cannot
run on the device without a compiler, so this package accepts either a
plain callable (sampled on the host into a table) or a ``Program``: per
channel, a list of segments (t_end, offset, amplitude, frequency, phase)
meaning offset + amplitude*cos(tau*frequency*t + phase) for t < t_end
(first matching segment), 0 after the last one.  That covers constant
fields, continuous-wave and chirp-free drives, pulse trains, Ramsey
sequences and piecewise-constant pulse shapes, evaluated on the GPU with
the same operation order as the host.
"""
import math

import numpy as np

CHANNELS = ("x", "y", "z", "r")


class Program:
    """Coefficient program of one trajectory (4 channels: x, y, z, r)."""

    def __init__(self, channels=None):
        self.channels = [list(c) for c in (channels or [[], [], [], []])]
        if len(self.channels) != 4:
            raise ValueError("a program has 4 channels: x, y, z, r")

    # -- building ---------------------------------------------------------
    def add(self, channel, t_end, offset=0.0, amplitude=0.0, frequency=0.0,
            phase=0.0):
        c = CHANNELS.index(channel) if isinstance(channel, str) else int(channel)
        self.channels[c].append((float(t_end), float(offset), float(amplitude),
                                 float(frequency), float(phase)))
        return self

    @classmethod
    def from_segments(cls, x=(), y=(), z=(), r=()):
        return cls([list(x), list(y), list(z), list(r)])

    # -- evaluation (host) -----------------------------------------------
    def value(self, channel, t):
        for t_end, off, amp, freq, ph in self.channels[channel]:
            if t < t_end:
                return off + amp*math.cos(math.tau*freq*t + ph)
        return 0.0

    def callables(self):
        """The four channel functions, as the reference's front end takes
        them."""
        return [lambda t, c=c: self.value(c, t) for c in range(4)]

    def as_array(self, nseg=None):
        """(4, nseg, 5) float64; unused segments never match (t_end=-inf)."""
        n = max(1, max(len(c) for c in self.channels))
        nseg = n if nseg is None else nseg
        if nseg < n:
            raise ValueError("nseg smaller than the longest channel")
        a = np.zeros((4, nseg, 5))
        a[:, :, 0] = -np.inf
        for c, segs in enumerate(self.channels):
            for s, seg in enumerate(segs):
                a[c, s] = seg
        return a

    def bound(self):
        """max |value| per channel."""
        return [max([abs(o) + abs(a) for _, o, a, _, _ in c] or [0.0])
                for c in self.channels]


def stack(programs):
    """(B, 4, S, 5) array from a list of Programs or (4, S, 5) arrays."""
    arrs = [p.as_array() if isinstance(p, Program) else np.asarray(p, dtype=np.float64)
            for p in programs]
    S = max(a.shape[1] for a in arrs)
    out = np.zeros((len(arrs), 4, S, 5))
    out[:, :, :, 0] = -np.inf
    for i, a in enumerate(arrs):
        out[i, :, :a.shape[1]] = a
    return out


def array_value(prog, channel, t):
    """Host evaluation of a (4, S, 5) program array at time t."""
    for t_end, off, amp, freq, ph in prog[channel]:
        if t < t_end:
            return off + amp*math.cos(math.tau*freq*t + ph)
    return 0.0
