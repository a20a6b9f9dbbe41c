"""Coefficient programs of common NV protocols, as (B, 4, S, 5) arrays for
``Sweep.run`` / ``sss_batch_run`` (channels x, y, z in tesla, r = optical
excitation as a fraction of saturation)."""
import numpy as np

GAMMA = 28.025e9     # Hz/T, the drive-amplitude convention of the workloads


def _empty(B, S):
    p = np.zeros((B, 4, S, 5))
    p[:, :, :, 0] = -np.inf
    return p


def odmr(freqs, rabi, laser):
    """Continuous drive b cos(2 pi f t) (b = rabi/GAMMA) with constant laser."""
    freqs = np.asarray(freqs, dtype=float)
    p = _empty(freqs.size, 1)
    p[:, :, 0, 0] = np.inf
    p[:, 0, 0, 2] = rabi/GAMMA
    p[:, 0, 0, 3] = freqs
    p[:, 3, 0, 1] = laser
    return p


def ramsey(rabi, detuning, tau, f_res, laser, t_init=1e-6, t_read=0.5e-6):
    """Laser initialisation, pi/2 - tau - pi/2 at frequency f_res + detuning
    (pulse length 1/(4 rabi)), laser readout.  Returns (programs, durations)."""
    rabi, detuning, tau = (np.asarray(a, dtype=float) for a in (rabi, detuning, tau))
    B = rabi.size
    p = _empty(B, 5)
    tp = 1/(4*rabi)
    e1 = t_init + tp
    e2 = e1 + tau
    e3 = e2 + tp
    end = e3 + t_read
    amp = rabi/GAMMA
    f = f_res + detuning
    for b in range(B):
        p[b, 0, 0] = (t_init, 0, 0, 0, 0)
        p[b, 0, 1] = (e1[b], 0, amp[b], f[b], 0)
        p[b, 0, 2] = (e2[b], 0, 0, 0, 0)
        p[b, 0, 3] = (e3[b], 0, amp[b], f[b], 0)
        p[b, 0, 4] = (np.inf, 0, 0, 0, 0)
        p[b, 3, 0] = (t_init, laser, 0, 0, 0)
        p[b, 3, 1] = (e3[b], 0, 0, 0, 0)
        p[b, 3, 2] = (np.inf, laser, 0, 0, 0)
    return p, end


def pulse_shapes(amplitudes, phases, seg_len, f_carrier, laser, t_read):
    """Piecewise-constant pulse shapes: segment s of shape b drives
    x = a cos(2 pi f t + phi), y = 0 ... as amplitude a_bs/GAMMA and phase
    phi_bs; then a laser readout of length t_read.  Returns (programs,
    durations)."""
    a = np.asarray(amplitudes, dtype=float)
    ph = np.asarray(phases, dtype=float)
    B, S = a.shape
    p = _empty(B, S + 1)
    for s in range(S):
        p[:, 0, s] = np.stack([np.full(B, (s + 1)*seg_len), np.zeros(B), a[:, s]/GAMMA,
                               np.full(B, f_carrier), ph[:, s]], axis=1)
    p[:, 0, S] = (np.inf, 0, 0, 0, 0)
    p[:, 3, 0] = (S*seg_len, 0, 0, 0, 0)
    p[:, 3, 1] = (np.inf, laser, 0, 0, 0)
    return p, np.full(B, S*seg_len + t_read)
