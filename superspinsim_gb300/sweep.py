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
    """A batched simulator for lab-frame generators (G, N, N).

    With ``use_rotating`` the batch runs in the reference's generalised
    rotating frame (``make_rotating`` of L0; simspins' default,
    superspinsim/sugar.py:536-558): the frame's step tables depend on the
    fine step, so ``time_step`` is needed up front, and ``run`` with another
    time step rebuilds the plan.  States, readout weights and results stay
    in the lab basis."""

    def __init__(self, generators, vectorisation_map=None, number_of_exponentials=2,
                 number_of_fine_divisions=1, lanes=0, cta_threads=0, variant=0,
                 use_rotating=False, time_step=None, use_residual=True):
        self.generators = np.ascontiguousarray(generators, dtype=np.float64)
        self.vectorisation_map = vectorisation_map
        self.N = self.generators.shape[1]
        self.F = int(number_of_fine_divisions)
        self.W, self.nodes = method(number_of_exponentials)
        self.residual = use_residual
        self._config = (lanes, cta_threads, variant)
        self.rotating = None
        if use_rotating:
            if time_step is None:
                raise ValueError("a rotating-frame sweep needs its time_step")
            from superspinsim_gb300.rotating import make_rotating
            new, V, Vi, d, s = make_rotating(self.generators[0], list(self.generators[1:]))
            self.rotating = dict(generators=np.array(new), vectors_real=V, inv_vectors_real=Vi,
                                 doubles=d, singles=s)
        self.time_step = None
        self._make_plan(time_step)

    def _make_plan(self, time_step):
        if self.rotating is None:
            self.plan = _lib.Plan(self.generators, self.W, self.nodes, residual=self.residual)
        else:
            from superspinsim_gb300.generate_simulator import rotating_tables
            r = self.rotating
            gn, dl, sl = rotating_tables(r["generators"], r["doubles"], r["singles"], self.nodes,
                                         time_step/self.F, self.residual)
            self.plan = _lib.Plan(None, self.W, self.nodes, residual=self.residual,
                                  rotating=dict(generators_nodes=gn, doubles_last=dl,
                                                singles_last=sl, vectors_real=r["vectors_real"],
                                                inv_vectors_real=r["inv_vectors_real"]))
        self.time_step = time_step
        self.plan.set_batch_config(*self._config)

    def flatten(self, rho0):
        rho0 = np.asarray(rho0)
        if rho0.ndim == 2 and rho0.shape[0] == rho0.shape[1] and rho0.shape[0] != self.N:
            rho0 = rho0[None]
        if rho0.shape[-1] == self.N and rho0.ndim == 2 and np.isrealobj(rho0):
            return np.ascontiguousarray(rho0, dtype=np.float64)
        return flatten_density(rho0, self.N, self.vectorisation_map)

    def run_sharded(self, rho0, programs, time_start, time_end, time_step, samples=None,
                    readout_weights=None, final_state=False, gather=True):
        """run() over the ranks of a multi-process job (one process per GPU,
        torchrun environment): each rank runs its contiguous range of the
        trajectories and, with gather, every rank receives the full
        readouts and final states in trajectory order.  No device
        collective; the host gather is the only exchange."""
        from superspinsim_gb300 import replicas
        if isinstance(programs, (list, tuple)):
            progs = list(programs)
        else:
            progs = np.ascontiguousarray(programs, dtype=np.float64)
        B = len(progs)
        flat = self.flatten(rho0)
        if flat.shape[0] == 1 and B > 1:
            flat = np.repeat(flat, B, axis=0)

        def runner(b, e):
            if e <= b:
                T = number_of_samples(time_start, time_end, time_step)
                out = {"time": time_start + time_step*(np.arange(T) + 1)}
                if readout_weights is not None:
                    out["readout"] = np.zeros((0, T))
                if final_state:
                    out["final"] = np.zeros((0, flat.shape[1]))
                return out
            return self.run(flat[b:e], progs[b:e], time_start, time_end, time_step,
                            samples=None if samples is None else np.asarray(samples)[b:e],
                            readout_weights=readout_weights, final_state=final_state)

        return replicas.run_sharded(runner, B, gather=gather)

    def run(self, rho0, programs, time_start, time_end, time_step, samples=None,
            readout_weights=None, final_state=False):
        """rho0: (B, n, n) complex or (B, N) flattened; programs: list of
        Program, (B, 4, S, 5), or a list of sampler callables
        ``sampler(time, row)`` (the reference's form, sampled on the host
        into a coefficient table).  Returns dict with 'time' (T,),
        'readout' (B, T) and 'final' (B, N) as requested."""
        T = number_of_samples(time_start, time_end, time_step)
        table = None
        if isinstance(programs, (list, tuple)) and programs and callable(programs[0]) \
                and not isinstance(programs[0], Program):
            table = self.sample(programs, time_start, time_step, T)
            progs = None
            B = table.shape[0]
        else:
            progs = stack(programs) if isinstance(programs, (list, tuple)) and \
                programs and isinstance(programs[0], Program) else \
                np.ascontiguousarray(programs, dtype=np.float64)
            B = progs.shape[0]
        flat = self.flatten(rho0)
        if flat.shape[0] == 1 and B > 1:
            flat = np.repeat(flat, B, axis=0)
        if self.rotating is not None and time_step != self.time_step:
            self._make_plan(time_step)
        ro, fin = self.plan.batch(flat, progs, time_start, time_step, T, self.F,
                                  samples=samples, readout_weights=readout_weights,
                                  want_final=final_state, table=table)
        out = {"time": time_start + time_step*(np.arange(T) + 1)}
        if ro is not None:
            out["readout"] = ro
        if fin is not None:
            out["final"] = fin
        return out

    def sample(self, samplers, time_start, time_step, T):
        """Coefficient tables (B, F*T*Q, G) of sampler callables, one per
        trajectory, in the row order of the batched table run (fine step
        r, sample t, node k): lab rows [c_L0, c_1, ...] (the reference's
        samplers write 1 for L0), rotating rows [c_1, ...]."""
        from superspinsim_gb300.generate_simulator import sample_table
        G = self.plan.G
        return np.concatenate([sample_table(s, G, time_start, time_step, T, self.F, self.nodes)
                               for s in samplers])

    def info(self):
        return self.plan.batch_info()


class ChunkedRun:
    """A prepared batch on the GPU, run in chunks of output samples.

    ``sss_batch_prepare`` analyses the batch once; every chunk is one
    ``sss_batch_launch`` that continues in place from the device state
    buffer, so a run can be stopped and resumed between chunks (``save`` /
    ``load``), and the sequence of chunk launches can be captured once in a
    CUDA graph and replayed (``replay``) for repeated sweeps whose inputs are
    refreshed in the same device buffers.  Device buffers are torch tensors.
    """

    def __init__(self, sweep, rho0, programs, time_start, time_step, T_max, samples=None,
                 readout_weights=None):
        import torch
        self.torch = torch
        self.sweep = sweep
        progs = stack(programs) if isinstance(programs, (list, tuple)) else np.ascontiguousarray(
            programs, dtype=np.float64)
        flat = sweep.flatten(rho0)
        if flat.shape[0] == 1 and progs.shape[0] > 1:
            flat = np.repeat(flat, progs.shape[0], axis=0)
        self.B, self.N = flat.shape
        self.t0, self.dt, self.T_max = float(time_start), float(time_step), int(T_max)
        dev = torch.device("cuda")
        self.rho0 = torch.from_numpy(np.ascontiguousarray(flat)).to(dev)
        self.state = self.rho0.clone()
        self.programs = torch.from_numpy(progs).to(dev)
        self.samples = None if samples is None else torch.from_numpy(
            np.ascontiguousarray(samples, dtype=np.int32)).to(dev)
        self.readout = None if readout_weights is None else torch.zeros(
            (self.B, self.T_max), dtype=torch.float64, device=dev)
        self.t_next = 0
        self.graph = None
        stream = torch.cuda.current_stream().cuda_stream
        # with uneven lengths the prepared batch also holds the layouts of
        # its later phases (wider lane groups as trajectories finish)
        sweep.plan.batch_prepare(self.rho0.data_ptr(), self.B, self.programs.data_ptr(),
                                 progs.shape[1], progs.shape[2], self.dt, sweep.F,
                                 readout_weights, stream=stream, samples=samples)

    def _launch(self, t_begin, n):
        self.sweep.plan.batch_launch(
            self.state.data_ptr(), self.programs.data_ptr(), self.t0, t_begin, n, self.T_max,
            samples_ptr=None if self.samples is None else self.samples.data_ptr(),
            readout_ptr=None if self.readout is None else self.readout.data_ptr(),
            stream=self.torch.cuda.current_stream().cuda_stream)

    def step(self, n_samples):
        """Run the next n_samples output samples (all trajectories)."""
        n = min(int(n_samples), self.T_max - self.t_next)
        if n > 0:
            self._launch(self.t_next, n)
            self.t_next += n
        return self.t_next

    def run(self, chunk=None):
        """Run the remaining samples in launches of `chunk` output samples
        (default: the autotuner's launch length for this sweep, else all
        remaining samples in one launch)."""
        chunk = chunk or getattr(self.sweep, "tuned_chunk", None) or self.T_max
        while self.t_next < self.T_max:
            self.step(chunk)
        return self

    def capture(self, chunk):
        """Capture the whole run, chunk by chunk, in one CUDA graph (the
        state starts again from rho0 on every replay)."""
        torch = self.torch
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side):
                self.state.copy_(self.rho0)
                for t in range(0, self.T_max, chunk):
                    self._launch(t, min(chunk, self.T_max - t))
        torch.cuda.current_stream().wait_stream(side)
        self.graph = g
        self.t_next = self.T_max
        return self

    def replay(self):
        self.graph.replay()
        return self

    def save(self, path):
        """Checkpoint: the device state, the next sample index, the batch
        shape and the readouts so far (omitted when the run has none)."""
        arrays = {"state": self.state.cpu().numpy(), "t_next": self.t_next,
                  "shape": np.array([self.B, self.N, self.T_max])}
        if self.readout is not None:
            arrays["readout"] = self.readout.cpu().numpy()
        np.savez(path, **arrays)

    def load(self, path):
        """Resume from a checkpoint written by save() for a batch of the same
        shape (plain arrays only: no pickled objects are read)."""
        with np.load(path, allow_pickle=False) as z:
            shape = tuple(int(v) for v in z["shape"])
            if shape != (self.B, self.N, self.T_max):
                raise ValueError(f"checkpoint is for (B, N, T_max) = {shape}, this run is "
                                 f"{(self.B, self.N, self.T_max)}")
            if (self.readout is not None) != ("readout" in z.files):
                raise ValueError("checkpoint and run disagree on whether readouts are kept")
            t_next = int(z["t_next"])
            if not 0 <= t_next <= self.T_max:
                raise ValueError(f"checkpoint sample index {t_next} out of range")
            self.state.copy_(self.torch.from_numpy(z["state"]))
            self.t_next = t_next
            if self.readout is not None:
                self.readout.copy_(self.torch.from_numpy(z["readout"]))
        return self

    def check(self):
        """Raise SSSError (ENONFINITE) if a chunk so far wrote a NaN or
        infinite readout or final state (waits for the current stream)."""
        self.sweep.plan.batch_check(self.torch.cuda.current_stream().cuda_stream)
        return self

    def results(self):
        self.check()
        out = {"final": self.state.cpu().numpy()}
        if self.readout is not None:
            out["readout"] = self.readout.cpu().numpy()
        return out
