"""Batched sweeps: many trajectories of one model in one call.

The reference has no batched API -- a parameter sweep calls ``simspins``
once per point, re-compiling everything each time (superspinsim/sugar.py:
566-583).  ``Sweep`` keeps one plan (device generators) and runs whole
batches through the persistent kernel of libsss.so: each trajectory has its
own coefficient program, initial state and length, and the kernel returns
a linear readout of the state after every output sample (for example the
excited-state population that gives NV fluorescence) plus the final states.
"""
import numpy as np

from superspinsim_gb300 import _lib
from superspinsim_gb300.generate_simulator import flatten_density, number_of_samples
from superspinsim_gb300.program import Program, stack
from superspinsim_gb300.quadratures import method


def population_weights(vectorisation_map, levels, scale=1.0):
    """Readout weights selecting the sum of the populations of `levels`
    (diagonal entries of the density matrix) in the flattened basis."""
    vm = np.asarray(vectorisation_map)
    w = np.zeros(vm.shape[0])
    for i, (y, x, c) in enumerate(vm):
        if y == x and c == 0 and int(y) in set(levels):
            w[i] = scale
    return w


def trapezoid(readout, dt, initial=None):
    """Integral of a readout trace sampled every dt starting at t0 + dt,
    with the value at t0 given by `initial` (trapezoid rule)."""
    r = np.asarray(readout)
    first = np.zeros(r.shape[:-1]) if initial is None else np.asarray(initial)
    return dt*(0.5*first + r[..., :-1].sum(axis=-1) + 0.5*r[..., -1])


class Sweep:
    """A batched simulator for lab-frame generators (G, N, N)."""

    def __init__(self, generators, vectorisation_map=None, number_of_exponentials=2,
                 number_of_fine_divisions=1, lanes=0, cta_threads=0, variant=0):
        self.generators = np.ascontiguousarray(generators, dtype=np.float64)
        self.vectorisation_map = vectorisation_map
        self.N = self.generators.shape[1]
        self.F = int(number_of_fine_divisions)
        W, nodes = method(number_of_exponentials)
        self.plan = _lib.Plan(self.generators, W, nodes)
        self.plan.set_batch_config(lanes, cta_threads, variant)

    def flatten(self, rho0):
        rho0 = np.asarray(rho0)
        if rho0.ndim == 2 and rho0.shape[0] == rho0.shape[1] and rho0.shape[0] != self.N:
            rho0 = rho0[None]
        if rho0.shape[-1] == self.N and rho0.ndim == 2 and np.isrealobj(rho0):
            return np.ascontiguousarray(rho0, dtype=np.float64)
        return flatten_density(rho0, self.N, self.vectorisation_map)

    def run(self, rho0, programs, time_start, time_end, time_step, samples=None,
            readout_weights=None, final_state=False):
        """rho0: (B, n, n) complex or (B, N) flattened; programs: list of
        Program or (B, 4, S, 5).  Returns dict with 'time' (T,), 'readout'
        (B, T) and 'final' (B, N) as requested."""
        progs = stack(programs) if isinstance(programs, (list, tuple)) and \
            programs and isinstance(programs[0], Program) else \
            np.ascontiguousarray(programs, dtype=np.float64)
        flat = self.flatten(rho0)
        if flat.shape[0] == 1 and progs.shape[0] > 1:
            flat = np.repeat(flat, progs.shape[0], axis=0)
        T = number_of_samples(time_start, time_end, time_step)
        ro, fin = self.plan.batch(flat, progs, time_start, time_step, T, self.F,
                                  samples=samples, readout_weights=readout_weights,
                                  want_final=final_state)
        out = {"time": time_start + time_step*(np.arange(T) + 1)}
        if ro is not None:
            out["readout"] = ro
        if fin is not None:
            out["final"] = fin
        return out

    def info(self):
        return self.plan.batch_info()
