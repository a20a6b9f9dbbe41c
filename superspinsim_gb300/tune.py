"""Autotuner for the batched kernel.

Times short prepared launches of the actual batch (a few output samples of
every trajectory) for each candidate configuration -- lanes per trajectory,
kernel variant (two FMA chains per row, one, row parts, packed slots or
phased row parts) and CTA size -- with CUDA events on the launch stream,
keeps the fastest, and then, for that configuration, times a window of
output samples run as launches of each candidate length (steps per launch,
in output samples of F fine steps): short launches give finer resume
points and graph chunks, long ones amortise the launch and the tail of
each launch.  The choice is cached per (model, batch size, fine steps) for
the process.
"""
import itertools

import numpy as np

from superspinsim_gb300.program import Program, stack

_CACHE = {}


def _key(sweep, B, progs):
    g = sweep.generators
    active = tuple(bool(np.any(progs[:, c, :, 1:3] != 0)) for c in range(progs.shape[1]))
    frame = None if getattr(sweep, "rotating", None) is None else sweep.time_step
    return (g.shape, float(np.abs(g).sum()), B, sweep.F, active, frame)


def autotune(sweep, rho0, programs, time_step, samples=None, probe_samples=2, repeats=2,
             lanes=(0, 8, 16, 32, 64, 128), variants=(1, 3, 4, 6, 7), threads=(32, 64, 128),
             chunks=(1, 4, 16, 64), chunk_tolerance=0.01, use_cache=True):
    """Pick and set the fastest batch configuration for this sweep and batch,
    then its launch length.  With uneven sample counts the lanes stay
    automatic (candidates other than 0 are dropped): a batch of uneven
    lengths runs in phases that widen the lane groups as trajectories
    finish, which only automatic lanes do, and probes of the first samples
    cannot see that gain.  Returns {"config": (lanes, variant, threads),
    "ms_per_traj_step": ..., "trials": [...], "samples_per_launch": c,
    "chunk_trials": [...]}: c is the shortest candidate launch length (in
    output samples) whose time over a window of max(chunks) samples is
    within chunk_tolerance of the best (chunks=() skips this stage; c is
    then None).  ChunkedRun.run uses it when given no chunk length."""
    import torch
    progs = stack(programs) if isinstance(programs, (list, tuple)) and programs and \
        isinstance(programs[0], Program) else np.ascontiguousarray(programs, dtype=np.float64)
    flat = sweep.flatten(rho0)
    if flat.shape[0] == 1 and progs.shape[0] > 1:
        flat = np.repeat(flat, progs.shape[0], axis=0)
    B = flat.shape[0]
    uneven = samples is not None and np.unique(np.asarray(samples)).size > 1
    if uneven:
        lanes = (0,)
    key = _key(sweep, B, progs) + (uneven,)
    if use_cache and key in _CACHE:
        best = _CACHE[key]
        L, var, th = best["config"]
        sweep.plan.set_batch_config(lanes=L, cta_threads=th, variant=var)
        sweep.tuned_chunk = best["samples_per_launch"]
        return best
    dev = torch.device("cuda")
    d_rho0 = torch.from_numpy(np.ascontiguousarray(flat)).to(dev)
    state = d_rho0.clone()
    d_prog = torch.from_numpy(progs).to(dev)
    stream = torch.cuda.current_stream()
    trials = []
    for L, var, th in itertools.product(lanes, variants, threads):
        if L and th % L:
            continue
        try:
            sweep.plan.set_batch_config(lanes=L, cta_threads=th, variant=var)
            sweep.plan.batch_prepare(d_rho0.data_ptr(), B, d_prog.data_ptr(), progs.shape[1],
                                     progs.shape[2], time_step, sweep.F,
                                     stream=stream.cuda_stream)
        except Exception as e:  # a configuration that does not fit
            trials.append({"config": (L, var, th), "error": str(e)})
            continue
        state.copy_(d_rho0)
        sweep.plan.batch_launch(state.data_ptr(), d_prog.data_ptr(), 0.0, 0, 1, probe_samples,
                                stream=stream.cuda_stream)
        times = []
        for _ in range(repeats):
            state.copy_(d_rho0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sweep.plan.batch_launch(state.data_ptr(), d_prog.data_ptr(), 0.0, 0, probe_samples,
                                    probe_samples, stream=stream.cuda_stream)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        info = sweep.plan.batch_info()
        trials.append({"config": (L, var, th), "ms": min(times), "lanes": info["lanes"]})
    ok = [t for t in trials if "ms" in t]
    if not ok:
        raise RuntimeError("no batch configuration fits: " + str(trials))
    best = min(ok, key=lambda t: t["ms"])
    steps = B*probe_samples*sweep.F
    result = {"config": best["config"], "ms_per_traj_step": best["ms"]/steps, "trials": trials,
              "samples_per_launch": None, "chunk_trials": []}
    L, var, th = best["config"]
    sweep.plan.set_batch_config(lanes=L, cta_threads=th, variant=var)
    if chunks:
        sweep.plan.batch_prepare(d_rho0.data_ptr(), B, d_prog.data_ptr(), progs.shape[1],
                                 progs.shape[2], time_step, sweep.F, stream=stream.cuda_stream)
        window = max(chunks)
        for c in sorted(chunks):
            times = []
            for _ in range(repeats):
                state.copy_(d_rho0)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for t in range(0, window, c):
                    sweep.plan.batch_launch(state.data_ptr(), d_prog.data_ptr(), 0.0, t,
                                            min(c, window - t), window,
                                            stream=stream.cuda_stream)
                e1.record(stream)
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
            result["chunk_trials"].append({"samples_per_launch": c, "launches": -(-window//c),
                                           "ms": min(times),
                                           "ms_per_traj_step": min(times)/(B*window*sweep.F)})
        fastest = min(t["ms"] for t in result["chunk_trials"])
        result["samples_per_launch"] = min(
            t["samples_per_launch"] for t in result["chunk_trials"]
            if t["ms"] <= fastest*(1 + chunk_tolerance))
    sweep.tuned_chunk = result["samples_per_launch"]
    _CACHE[key] = result
    return result
