"""Gradients of time-integrated readouts with respect to drive pulses.

``sss_adjoint_run`` (libsss.so) computes, for a batch of trajectories, the
objective J = sum_t tw[t] * rw . rho(t) -- e.g. integrated fluorescence --
and its gradient with respect to the amplitude and phase of every segment
of the x-drive channel (``sss_adjoint_run_channel``: amplitude, phase,
offset and frequency of the segments of any channel, such as a detuned y
drive or the laser power), by an adjoint sweep on the GPU: the forward pass
stores the state before every exponential when device memory allows it
(trajectories in memory-sized chunks) and the backward pass walks the
stored states; when one trajectory's states do not fit, a checkpointed
sweep (about sqrt(steps) checkpoints, each interval recomputed) runs
instead.
``PulseObjective`` exposes it to torch.autograd: piecewise-constant pulse
amplitudes (Rabi frequency, Hz) and phases (rad) in, objective out.
"""
import numpy as np

from superspinsim_gb300 import _lib, protocols
from superspinsim_gb300.generate_simulator import flatten_density
from superspinsim_gb300.quadratures import method
from superspinsim_gb300.sweep import population_weights


def trapezoid_weights(T, dt, first, last):
    """Time weights of the trapezoid rule over output samples first..last
    (inclusive; sample t is at t0 + dt*(t+1))."""
    w = np.zeros(T)
    if last > first:
        w[first:last + 1] = dt
        w[first] = w[last] = dt/2
    return w


class Objective:
    """A fixed model and readout; evaluates J and dJ/d(pulse) for batches."""

    def __init__(self, generators, vectorisation_map, rho0, readout_levels, readout_rate,
                 number_of_exponentials=2, number_of_fine_divisions=200):
        self.gens = np.ascontiguousarray(generators, dtype=np.float64)
        self.vm = vectorisation_map
        N = self.gens.shape[1]
        self.rho0 = flatten_density(rho0, N, vectorisation_map)
        self.rw = population_weights(vectorisation_map, readout_levels, readout_rate)
        self.F = number_of_fine_divisions
        W, nodes = method(number_of_exponentials)
        self.plan = _lib.Plan(self.gens, W, nodes)

    def run(self, programs, dt, T, time_weights, channel=None):
        """J (B,) and gradient (B, nseg, 2) w.r.t. (amplitude [program
        units], phase) of every x-channel segment; with `channel`, the
        gradient (B, nseg, 4) w.r.t. (amplitude, phase, offset, frequency)
        of that channel's segments."""
        B = programs.shape[0]
        rho0 = np.repeat(self.rho0[None], B, axis=0)
        if channel is not None:
            return self.plan.adjoint_channel(rho0, programs, 0.0, dt, T, self.F, self.rw,
                                             time_weights, channel)
        return self.plan.adjoint(rho0, programs, 0.0, dt, T, self.F, self.rw, time_weights)

    def forward_only(self, programs, dt, T, time_weights):
        """J from the batched forward kernel (no gradient)."""
        B = programs.shape[0]
        rho0 = np.repeat(self.rho0[None], B, axis=0)
        ro, _ = self.plan.batch(rho0, programs, 0.0, dt, T, self.F, readout_weights=self.rw)
        return ro @ time_weights


def make_pulse_function(objective, seg_len, f_carrier, laser, t_read, dt):
    """A torch.autograd.Function computing J for pulse shapes
    (amplitudes as Rabi frequencies in Hz, phases in rad), each shape a row."""
    import torch

    class PulseObjective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, rabi, phase):
            a = rabi.detach().cpu().numpy().astype(np.float64)
            p = phase.detach().cpu().numpy().astype(np.float64)
            progs, dur = protocols.pulse_shapes(a, p, seg_len, f_carrier, laser, t_read)
            T = int(round(dur[0]/dt))
            S = a.shape[1]
            tw = trapezoid_weights(T, dt, int(round(S*seg_len/dt)) - 1, T - 1)
            J, grad = objective.run(progs, dt, T, tw)
            g = torch.from_numpy(grad[:, :S]).to(rabi.device)
            # program amplitude = rabi/GAMMA
            ctx.save_for_backward(g[..., 0]/protocols.GAMMA, g[..., 1])
            return torch.from_numpy(J).to(rabi.device)

        @staticmethod
        def backward(ctx, gJ):
            ga, gp = ctx.saved_tensors
            return gJ[:, None]*ga, gJ[:, None]*gp

    return PulseObjective
