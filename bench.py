"""Throughput benchmark: the 7-level NV ODMR sweep.

Workload (one bench step): 1024 microwave frequencies uniform over
+-30 MHz around the ms=0 -> +1 resonance of the 7-level NV model (ground
D = 2.870 GHz, excited D = 1.42 GHz, B = 5 mT along z, optical decay
65.9 /us, ISC 11 /us and 80 /us, singlet decay 3.0 /us and 2.6 /us), Rabi
5 MHz, laser pumping 10 /us; each trajectory 2 us at dt = 5 ps with the
4th-order commutator-free Magnus method (CF4:2), 400,000 steps, readout
of the excited-state population every 1 ns (T = 2000, F = 200), vectorised
density of length 49 (Liouvillian 49 x 49, float64).  Unit: trajectory
steps per second, one trajectory step = one CF4:2 step of one trajectory.

Arms:
  default           the batched persistent kernel of libsss.so.  `value`
                    times sss_batch_run on device-resident inputs; `e2e`
                    times the public API (superspinsim_gb300.sweep.Sweep.run)
                    from host buffers to host readouts.
  --impl reference  the reference's algorithm on the host cores: the CPU
                    oracle (a C/OpenMP restatement of the reference's
                    simulate -- 2R = 70 dense squarings per exponential,
                    serial chain of step propagators) on a bounded sample
                    of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N_FREQ = 1024
DURATION = 2e-6
DT_OUT = 1e-9
F = 200
K_EXP = 2
B_FIELD = 5e-3
GAMMA = 28.025e9
F_RES = 2.870e9 + GAMMA*B_FIELD
RABI = 5e6
LASER = 10/65.9
METRIC = "NV-7 ODMR traj-steps/s"


def nv7_model():
    """Generators (5, 49, 49) and vectorisation map of the 7-level NV at
    B = 5 mT with the workload's rates."""
    from superspinsim_gb300 import models
    from superspinsim_gb300.generators import generate_atoms
    spins, inter, groups = models.nv_7(np.array([0.0, 0.0, B_FIELD]),
                                       params=models.odmr_params())
    g, vm = generate_atoms(spins, inter, groups, use_incoherent=False)
    gens = np.array([g["generators"][k] for k in ("L0", "Gx", "Gy", "Gz", "Gr")])
    return gens, vm


def workload(n_freq=N_FREQ):
    freqs = F_RES + np.linspace(-30e6, 30e6, n_freq)
    progs = np.zeros((n_freq, 4, 1, 5))
    progs[:, :, :, 0] = np.inf
    progs[:, 0, 0, 2] = RABI/GAMMA
    progs[:, 0, 0, 3] = freqs
    progs[:, 3, 0, 1] = LASER
    rho = np.zeros((7, 7), complex)
    rho[1, 1] = 1.0
    return progs, rho


def build_workload(name, args):
    """(generators, vmap, programs (B,4,S,5), rho (n,n), samples or None,
    T_max, readout levels, description dict)."""
    from superspinsim_gb300 import models, protocols
    from superspinsim_gb300.generators import generate_atoms
    if name == "odmr":
        gens, vm = nv7_model()
        progs, rho = workload(args.n_freq)
        T = int(round(args.duration/DT_OUT))
        desc = {"workload": "NV-7 ODMR sweep, 1024 frequencies x 2 us at 5 ps "
                            "(400k CF4:2 steps each), readout every 1 ns",
                "n_freq": progs.shape[0], "n_levels": 7, "liouvillian": "49x49"}
        return gens, vm, progs, rho, None, T, [3, 4, 5], desc
    if name == "ramsey":
        gens, vm = nv7_model()
        rng = np.random.default_rng(20260103)
        B = args.n_traj or 4096
        rabi = rng.uniform(2e6, 10e6, B)
        det = rng.uniform(-5e6, 5e6, B)
        tau = rng.uniform(0, 5e-6, B)
        progs, dur = protocols.ramsey(rabi, det, tau, F_RES, LASER)
        samples = np.ceil(dur/DT_OUT).astype(np.int32)
        rho = np.zeros((7, 7), complex)
        rho[1, 1] = 1.0
        desc = {"workload": f"NV-7 Ramsey, {B} seeded trajectories (Rabi 2-10 MHz, detuning "
                            "+-5 MHz, tau 0-5 us; laser 1 us, pi/2, tau, pi/2, laser 0.5 us) "
                            "at 5 ps, uneven lengths",
                "n_traj": B, "n_levels": 7, "liouvillian": "49x49",
                "traj_steps_total": int(samples.sum())*F}
        return gens, vm, progs, rho, samples, int(samples.max()), [3, 4, 5], desc
    if name == "nv21":
        spins, inter, groups = models.nv_21(np.array([0.0, 0.0, 0.05]),
                                            params=models.nv21_params())
        g, vm = generate_atoms(spins, inter, groups, use_incoherent=False)
        gens = np.array([g["generators"][k] for k in ("L0", "Gx", "Gy", "Gz", "Gr")])
        B = args.n_traj or 256
        f_res = 2.870e9 + GAMMA*0.05
        progs = protocols.odmr(f_res + np.linspace(-30e6, 30e6, B), RABI, LASER)
        rho = np.zeros((21, 21), complex)
        for k in range(3, 6):
            rho[k, k] = 1/3
        T = int(round(args.duration/DT_OUT)) if args.duration != DURATION else 1000
        desc = {"workload": f"NV-21 (NV + 14N) ODMR sweep, {B} frequencies x {T} ns at 5 ps",
                "n_freq": B, "n_levels": 21, "liouvillian": "441x441"}
        return gens, vm, progs, rho, None, T, list(range(9, 18)), desc
    raise ValueError(name)


class ClockSampler:
    """nvidia-smi clock/throttle samples taken while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0] or None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        _ = dev
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    from superspinsim_gb300 import replicas
    return replicas.init()


def barrier(world):
    if world > 1:
        from superspinsim_gb300 import replicas
        replicas.barrier()


def max_over_ranks(x, world):
    from superspinsim_gb300 import replicas
    return replicas.max_over_ranks(x) if world > 1 else x


def executed_flops_per_traj_step(info, K):
    """FP64 flops one trajectory step of the batched kernel computes: per
    exponential, the assembly of the generators whose coefficient varies on
    their non-zeros of the pruned pattern (2 live_nnz; the constant ones are
    a precomputed table), and per sub-step d Taylor terms of 2 flops per
    non-zero and 2 per row (its v term) plus one multiply per row (the
    scaled form's 1/d!)."""
    nnz, rows, d, m = info["nnz"], info["rows"], info["degree"], info["substeps"]
    return K*(2*info["live_nnz"] + m*(d*(2*nnz + 2*rows) + rows))


def dense_flops_per_traj_step(N, G, K, m):
    """The dense formula K (2 G N^2 + m 2 N^3 + 2 N^2) with m matrix products
    per exponential, for comparison (the reference's scheme has m = 70)."""
    return K*(2*G*N*N + m*2*N**3 + 2*N*N)


def fp64_issue_per_traj_step(info, K, L):
    """FP64 warp instructions one trajectory step issues (its share of its
    group's instructions): d terms of fp64_per_term instructions per
    exponential and sub-step, over the 32/L trajectories of a warp."""
    per_group = K*info["substeps"]*info["degree"]*info["fp64_per_term"]
    return per_group*min(L, 32)/32


CPU_SAMPLES = 16   # output samples of the bounded CPU sample (x F fine steps)


def full_length_parity(plan, N):
    """The workload's trajectory nearest the ms=0 -> +1 line over all
    400,000 steps through the batched kernel (the layout the bench chose),
    against the reference's own algorithm: the fixture of the oracle's
    reference mode (70 squarings per exponential), tests/golden/
    nv7_fullrun.npz.  Density max-abs at every 100th sample and the
    fluorescence at every sample."""
    path = os.path.join(ROOT, "tests", "golden", "nv7_fullrun.npz")
    with np.load(path) as z:
        fx = {k: z[k] for k in z.files}
    T, dt, Fx = int(fx["T"]), float(fx["dt"]), int(fx["F"])
    ro, _, tr = plan.batch(fx["rho0"][None], fx["program"][None], 0.0, dt, T, Fx,
                           readout_weights=fx["readout_weights"], want_trace=True)
    ref_f = fx["fluorescence"]
    return {"vs": "the reference's algorithm (oracle reference mode, 70 squarings per "
                  "exponential) on the sweep's trajectory nearest resonance, all 400,000 "
                  "steps (tests/golden/nv7_fullrun.npz)",
            "density_max_abs": float(np.abs(tr[0][fx["kept_samples"]] - fx["states"]).max()),
            "fluorescence_rel_max": float(np.abs(ro[0] - ref_f).max()/np.abs(ref_f).max()),
            "bars": {"density_max_abs": 1e-10, "fluorescence_rel": 1e-9}}


def cpu_vector_baseline(threads=0, n_freq=N_FREQ, n_traj=64, T_s=64):
    """The batched kernel's own algorithm on the host cores (the CPU
    oracle's vector mode: the sparse Taylor action, degree 16) on a bounded
    sample of the workload: its first n_traj trajectories for T_s output
    samples of F = 200 steps, trajectories spread over the cores."""
    from oracle import oracle
    from superspinsim_gb300.quadratures import method
    gens, vm = nv7_model()
    progs, rho = workload(n_freq)
    W, nodes = method(K_EXP)
    t = time.perf_counter()
    oracle.simulate(gens, np.stack([rho]*n_traj), 0.0, T_s*DT_OUT + DT_OUT*1e-4, DT_OUT,
                    progs[:n_traj], K=K_EXP, W=W, nodes=nodes, F=F, vectorisation_map=vm,
                    mode="vector", degree=16, threads=threads, flat_out=True)
    el = time.perf_counter() - t
    n = n_traj*T_s*F
    return {"value": n/el, "unit": "traj-steps/s", "cores": threads or oracle.max_threads(),
            "kind": "port",
            "sample": f"trajectories 0-{n_traj - 1} of the workload, {T_s} samples x F={F} "
                      f"each ({n} CF4:2 steps), the batched kernel's algorithm (sparse Taylor "
                      f"action on the reachable pattern)"}


def cpu_baseline(steps=None, threads=0, n_freq=N_FREQ):
    """The reference's algorithm (CPU oracle, reference mode) on a bounded
    sample of the workload: its trajectory 0 for 16 output samples of F =
    200 fine steps at 5 ps (3200 trajectory steps), on all host cores
    (OpenMP over output samples).  Also returns the flattened states after
    every sample (key "states"), the reference result of the parity check."""
    from oracle import oracle
    from superspinsim_gb300.quadratures import method
    gens, vm = nv7_model()
    progs, rho = workload(n_freq)
    W, nodes = method(K_EXP)
    T_s = CPU_SAMPLES
    t = time.perf_counter()
    _, states = oracle.simulate(gens, rho, 0.0, T_s*DT_OUT + DT_OUT*1e-4, DT_OUT, progs[0],
                                K=K_EXP, W=W, nodes=nodes, F=F, R=35, residual=True,
                                vectorisation_map=vm, mode="reference", threads=threads,
                                flat_out=True)
    el = time.perf_counter() - t
    n = T_s*F
    return {"value": n/el, "unit": "traj-steps/s",
            "cores": threads or oracle.max_threads(), "kind": "port",
            "sample": f"trajectory 0 of the workload, {n} CF4:2 steps ({T_s} samples x F={F}), "
                      f"reference algorithm (70 squarings per exponential)",
            "seconds": el, "states": states}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    samples = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline()
        if i >= args.warmup:
            samples.append(r)
    total_steps = sum(r["value"]*r["seconds"] for r in samples)
    total_time = sum(r["seconds"] for r in samples)
    v = total_steps/total_time
    cb = dict(samples[0])
    cb["value"] = v
    cb.pop("seconds", None)
    cb.pop("states", None)
    line = {"metric": METRIC, "value": v, "unit": "traj-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3*total_time/args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {**build_workload("odmr", args)[-1], "frame": "lab", "method": "CF4:2",
                       "dt_s": DT_OUT/F, "samples": int(round(args.duration/DT_OUT)),
                       "fine_divisions": F, "parallelism": "host cores",
                       "sample": cb["sample"]},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "traj-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def adjoint_workload(nv21=False, n_traj=0, n_seg=0, readout=300e-9):
    """Pulse-shape objective of the adjoint workloads: NV-7 at 5 mT, 256
    seeded shapes of 128 piecewise-constant segments of 2 ns (Rabi 0-20 MHz,
    phase 0-2pi, carrier at the ms=0 -> +1 line), or NV-21 (14N) at 50 mT,
    32 shapes of 64 segments; each followed by a 300 ns laser readout whose
    integrated fluorescence is the objective.  Returns (Objective, programs
    (B,4,S,5), T, time weights, S, name)."""
    from superspinsim_gb300 import protocols
    from superspinsim_gb300.adjoint import Objective, trapezoid_weights
    if nv21:
        from superspinsim_gb300 import models
        from superspinsim_gb300.generators import generate_atoms
        spins, inter, groups = models.nv_21(np.array([0.0, 0.0, 0.05]),
                                            params=models.nv21_params())
        g, vm = generate_atoms(spins, inter, groups, use_incoherent=False)
        gens = np.array([g["generators"][k] for k in ("L0", "Gx", "Gy", "Gz", "Gr")])
        B, S, f_c = n_traj or 32, n_seg or 64, 2.870e9 + GAMMA*0.05
        rho = np.zeros((21, 21), complex)
        for k in range(3, 6):
            rho[k, k] = 1/3
        levels = list(range(9, 18))
    else:
        gens, vm = nv7_model()
        B, S, f_c = n_traj or 256, n_seg or 128, F_RES
        rho = np.zeros((7, 7), complex)
        rho[1, 1] = 1.0
        levels = [3, 4, 5]
    rng = np.random.default_rng(20260104)
    rabi = rng.uniform(0, 20e6, (B, S))
    phase = rng.uniform(0, 2*np.pi, (B, S))
    progs, dur = protocols.pulse_shapes(rabi, phase, 2e-9, f_c, LASER, readout)
    T = int(round(dur[0]/DT_OUT))
    tw = trapezoid_weights(T, DT_OUT, S*2 - 1, T - 1)
    obj = Objective(gens, vm, rho, levels, 65.9e6, number_of_exponentials=K_EXP,
                    number_of_fine_divisions=F)
    return obj, progs, T, tw, S, "NV-21" if nv21 else "NV-7"


def adjoint_measurement(steps=2, warmup=1):
    """The adjoint half of the metric on its workload (NV-7, 256 pulse shapes
    x 128 segments, 256 parameters each): gradients/s, the ratio to one
    forward solve, and four gradient entries of one shape against central
    differences of the GPU forward with h = 1e-6 (relative for amplitudes),
    with the clocks sampled while it runs."""
    import torch
    obj, progs, T, tw, S, name = adjoint_workload(False)
    B = progs.shape[0]
    for _ in range(warmup):
        obj.run(progs, DT_OUT, T, tw)
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    fwd, adj = [], []
    for _ in range(steps):
        t = time.perf_counter()
        obj.forward_only(progs, DT_OUT, T, tw)
        fwd.append(time.perf_counter() - t)
        t = time.perf_counter()
        J, grad = obj.run(progs, DT_OUT, T, tw)
        adj.append(time.perf_counter() - t)
    clock_info = clocks.stop()
    fwd_s, adj_s = statistics.median(fwd), statistics.median(adj)
    b = 1
    pert, idx = [], []
    for seg in (0, S//2):
        for comp, col in ((0, 2), (1, 4)):
            h = 1e-6*progs[b, 0, seg, 2] if comp == 0 else 1e-6
            for step in (h, -h):
                pp = progs[b].copy()
                pp[0, seg, col] += step
                pert.append(pp)
            idx.append((seg, comp, h))
    Jp = obj.forward_only(np.stack(pert), DT_OUT, T, tw)
    errs = []
    for k, (seg, comp, h) in enumerate(idx):
        fd = (Jp[2*k] - Jp[2*k + 1])/(2*h)
        errs.append(abs(grad[b, seg, comp] - fd)/max(abs(fd), 1e-300))
    return {"value": B/adj_s, "unit": f"gradients/s ({2*S} parameters each)",
            "workload": f"{name}, {B} pulse shapes x {S} segments of 2 ns + 300 ns laser "
                        f"readout, dt 5 ps ({T*F:,} steps each); objective: integrated "
                        f"fluorescence over the readout",
            "ms_per_gradient_batch": 1e3*adj_s, "adjoint_over_forward": adj_s/fwd_s,
            "forward_traj_steps_per_s": B*T*F/fwd_s,
            "fd_check": {"shape": b, "entries": len(errs), "h": 1e-6,
                         "rel_err_max": float(max(errs))},
            "clocks": clock_info}


def run_adjoint_workload(args, rank, world):
    """Times the checkpointed adjoint (objective + 2S gradients per shape)
    of adjoint_workload against one forward solve of the same batch."""
    import torch
    obj, progs, T, tw, S, name = adjoint_workload(args.workload == "adjoint-nv21", args.n_traj,
                                                  args.segments, args.readout)
    B = progs.shape[0]
    for _ in range(args.warmup):
        obj.run(progs, DT_OUT, T, tw)
    torch.cuda.synchronize()
    fwd, adj = [], []
    for _ in range(args.steps):
        t = time.perf_counter()
        obj.forward_only(progs, DT_OUT, T, tw)
        fwd.append(time.perf_counter() - t)
        t = time.perf_counter()
        J, grad = obj.run(progs, DT_OUT, T, tw)
        adj.append(time.perf_counter() - t)
    fwd_s, adj_s = statistics.median(fwd), statistics.median(adj)
    steps = B*T*F
    line = {"metric": f"{name} pulse-shape adjoint gradients/s", "value": B/adj_s,
            "unit": f"gradients/s ({2*S} parameters each)", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3*adj_s, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{B} pulse shapes x {S} segments of 2 ns + "
                                   f"{args.readout*1e9:g} ns readout, {name}, dt 5 ps "
                                   f"({T*F:,} steps each)",
                       "parameters_per_shape": 2*S, "traj_steps": steps},
            "adjoint_over_forward": adj_s/fwd_s,
            "forward_traj_steps_per_s": steps/fwd_s,
            "adjoint_traj_steps_per_s": steps/adj_s,
            "objective_mean": float(np.mean(J))}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-freq", type=int, default=N_FREQ)
    ap.add_argument("--duration", type=float, default=DURATION)
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--variant", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="odmr",
                    choices=["odmr", "ramsey", "nv21", "adjoint", "adjoint-nv21"])
    ap.add_argument("--n-traj", type=int, default=0)
    ap.add_argument("--segments", type=int, default=0,
                    help="adjoint workloads: pulse segments per shape (default 128, NV-21 64)")
    ap.add_argument("--readout", type=float, default=300e-9,
                    help="adjoint workloads: laser readout after the pulses (s)")
    ap.add_argument("--graph-chunk", type=int, default=0,
                    help="time a CUDA graph of the prepared run in chunks of this many output "
                         "samples (resumable launches) instead of one launch")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the adjoint measurement of the default line")
    ap.add_argument("--rotating", action="store_true",
                    help="run the batch in the generalised rotating frame (simspins' default)")
    args = ap.parse_args()
    rank, world = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return
    if args.workload in ("adjoint", "adjoint-nv21"):
        run_adjoint_workload(args, rank, world)
        return

    import torch
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.generate_simulator import flatten_density
    from superspinsim_gb300.sweep import Sweep, population_weights, trapezoid

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    gens, vm, progs_all, rho, samples_all, T, levels, wdesc = build_workload(args.workload, args)
    N = vm.shape[0]
    B_all = progs_all.shape[0]
    # the sweep's trajectories are sharded over the ranks (contiguous ranges,
    # no device collective); the job's units are the whole sweep's
    from superspinsim_gb300 import replicas
    t_begin, t_end = replicas.shard(B_all, rank, world)
    progs = progs_all[t_begin:t_end]
    samples = None if samples_all is None else samples_all[t_begin:t_end]
    B = progs.shape[0]
    units_per_step = int(samples_all.sum())*F if samples_all is not None else B_all*T*F
    rho0 = np.repeat(flatten_density(rho, N, vm)[None], B, axis=0)
    w = population_weights(vm, levels)
    sweep = Sweep(gens, vm, number_of_exponentials=K_EXP, number_of_fine_divisions=F,
                  lanes=args.lanes, cta_threads=args.threads, variant=args.variant,
                  use_rotating=args.rotating, time_step=DT_OUT)
    wdesc["frame"] = "rotating" if args.rotating else "lab"
    plan = sweep.plan
    tuned = None
    if not (args.lanes or args.threads or args.variant):
        from superspinsim_gb300.tune import autotune
        tuned = autotune(sweep, rho0, progs, DT_OUT, samples=samples)

    stream = torch.cuda.Stream()
    d_rho0 = torch.from_numpy(rho0).cuda()
    d_prog = torch.from_numpy(progs).cuda()
    d_smp = torch.from_numpy(samples).cuda() if samples is not None else None
    d_ro = torch.empty((B, T), dtype=torch.float64, device="cuda")
    flush = torch.empty(256*1024*1024//4, dtype=torch.float32, device="cuda")  # > L2

    def step():
        plan.batch_device(d_rho0.data_ptr(), B, d_prog.data_ptr(), 4, progs.shape[2], 0.0,
                          DT_OUT, T, F,
                          samples_ptr=d_smp.data_ptr() if d_smp is not None else None,
                          readout_weights=w, readout_ptr=d_ro.data_ptr(),
                          stream=stream.cuda_stream)

    n_chunks = 0
    if args.graph_chunk:
        # the prepared batch in chunks of output samples, captured once in a
        # CUDA graph; a step is one replay (state reset + every chunk launch)
        from superspinsim_gb300.sweep import ChunkedRun
        with torch.cuda.stream(stream):
            chunked = ChunkedRun(sweep, rho0, progs, 0.0, DT_OUT, T, samples=samples,
                                 readout_weights=w).capture(args.graph_chunk)
        n_chunks = -(-T//args.graph_chunk)
        wdesc["chunks"] = {"samples_per_chunk": args.graph_chunk, "launches_per_step": n_chunks,
                           "cuda_graph": True}

        def step():  # noqa: F811
            chunked.replay()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        clocks = ClockSampler()
        clocks.start()
        times, kernel_ms = [], []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            barrier(world)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
            kernel_ms.append(0.0 if n_chunks else plan.batch_info()["kernel_ms"])
        barrier(world)
        clock_info = clocks.stop()
    # every readout the timed steps wrote was finite (raises otherwise)
    plan.batch_check(stream.cuda_stream)
    info = plan.batch_info()
    launches = (n_chunks or plan.last_launches())*args.steps
    total_ms = max_over_ranks(sum(times), world)
    units = units_per_step*args.steps
    value = units/(total_ms/1e3)

    # e2e: public API, host buffers in and out, every step
    e2e_times = []
    for i in range(1 + args.steps):  # the plan and kernel are already warm
        torch.cuda.synchronize()
        barrier(world)
        t = time.perf_counter()
        out = sweep.run_sharded(np.repeat(rho[None], B_all, axis=0), progs_all, 0.0,
                                T*DT_OUT + 1e-13, DT_OUT, samples=samples_all, readout_weights=w)
        fluor = 65.9e6*trapezoid(out["readout"], DT_OUT)
        el = time.perf_counter() - t
        if i >= 1:
            e2e_times.append(el)
    e2e_s = max_over_ranks(sum(e2e_times), world)
    e2e_value = units_per_step*args.steps/e2e_s
    h2d = rho0.nbytes + progs.nbytes + (samples.nbytes if samples is not None else 0)
    d2h = B*T*8

    # the plain per-trajectory drop-in (generate_simulator / simulate) on a
    # subset of the same workload: 1 trajectory, 64 output samples
    from superspinsim_gb300 import generate_simulator
    plain_value = None
    if N <= 52:
        plain_sim = generate_simulator(progs[0], gens, vm, number_of_exponentials=K_EXP,
                                       number_of_fine_divisions=F)
        plain_T = T  # one whole trajectory: T step-propagator CTAs fill the GPU
        plain_sim(rho, 0.0, 8*DT_OUT + 1e-13, DT_OUT)
        torch.cuda.synchronize()
        t = time.perf_counter()
        plain_sim(rho, 0.0, plain_T*DT_OUT + 1e-13, DT_OUT)
        plain_s = time.perf_counter() - t
        plain_value = plain_T*F/plain_s

    fl = executed_flops_per_traj_step(info, K_EXP)
    issue = fp64_issue_per_traj_step(info, K_EXP, info["lanes"])
    # the kernel's device time per step: the launch's own events, or with
    # graph chunks (events of the last chunk only) the step's event time
    kms = statistics.mean(kernel_ms) if not n_chunks else statistics.mean(times)
    local_units = (int(samples.sum())*F if samples is not None else B*T*F)
    achieved = fl*local_units/(kms*1e-3)/1e12
    peak = _lib.fp64_peak_tflops()
    mma_peak = _lib.fp64_mma_peak_tflops()
    # FP64 warp-instruction slots of the GPU per second at the peak rate
    # (the peak's FMAs per second over 32 lanes)
    issue_peak = peak*1e12/2/32
    # algorithmic DRAM bytes of one launch: initial states and programs read
    # once, readouts written once
    traffic = rho0.nbytes + progs.nbytes + B*T*8 + (samples.nbytes if samples is not None else 0)
    line = {"metric": METRIC, "value": value, "unit": "traj-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms/args.steps,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {**wdesc, "method": "CF4:2",
                       "dt_s": DT_OUT/F, "samples": T, "fine_divisions": F,
                       "traj_steps_per_step": units_per_step,
                       "l2": "flushed between timed steps (256 MiB write)",
                       "autotune": None if tuned is None else {
                           "chosen": {"lanes": tuned["config"][0], "variant": tuned["config"][1],
                                      "cta_threads": tuned["config"][2]},
                           "trials": len(tuned["trials"]),
                           "samples_per_launch": tuned["samples_per_launch"],
                           "launch_length_trials": {
                               str(t["samples_per_launch"]): round(t["ms_per_traj_step"]*1e6, 5)
                               for t in tuned["chunk_trials"]},
                           "launch_length_unit": "ns per traj-step over a 64-sample window"},
                       "kernel": {"lanes": info["lanes"], "taylor_degree": info["degree"],
                                  "substeps": info["substeps"], "rows": info["rows"],
                                  "nnz": info["nnz"], "variant": info["variant"],
                                  "live_generators": info["live_generators"],
                                  "live_nnz": info["live_nnz"],
                                  "fp64_per_horner_term": info["fp64_per_term"],
                                  "bank_extra_wavefronts_per_term":
                                      info["bank_extra_wavefronts_per_term"],
                                  # uneven lengths run in phases of widening lane
                                  # groups; "lanes" is the last phase's
                                  "launches_per_run": n_chunks or plan.last_launches()},
                       "parallelism": f"trajectory shards x{world}"},
            "e2e": {"value": e2e_value, "unit": "traj-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "plain_dropin": None if plain_value is None else {
                "value": plain_value, "unit": "traj-steps/s",
                "sample": f"generate_simulator/simulate, 1 trajectory x "
                          f"{plain_T*F} steps of the workload",
                "batched_over_plain": value/plain_value},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved/peak,
                         "traffic": traffic,
                         "traffic_note": "bytes of one launch: initial states and programs "
                                         "read once, readouts written once (the kernel keeps "
                                         "its working set in shared memory; an ncu capture of "
                                         "the same kernel at 20 samples read 630 B of DRAM, "
                                         "its 0.16 MB of readouts staying in L2)",
                         "peak_source": "measured live (sss_fp64_peak DFMA loop)",
                         "flops_note": "executed: assembly of the drive generators on their "
                                       "non-zeros, d Taylor terms of 2 flops per non-zero "
                                       "and per row, 1/d! per row",
                         "fp64_issue": {"per_traj_step": issue,
                                        "achieved_per_s": issue*local_units/(kms*1e-3),
                                        "peak_per_s": issue_peak,
                                        "frac": issue*local_units/(kms*1e-3)/issue_peak,
                                        "note": "FP64 warp instructions issued (lanes of a "
                                                "warp instruction not carrying a flop count "
                                                "here but not in `achieved`)"},
                         "dense_formula_flops_per_traj_step": {
                             "m_70": dense_flops_per_traj_step(N, gens.shape[0], K_EXP, 70),
                             "note": "the reference's scheme, K (2 G N^2 + 70 x 2 N^3 + 2 N^2)"},
                         "fp64_tensor": {"dmma_peak": mma_peak, "unit": "TFLOP/s",
                                         "used": False,
                                         "note": "measured live (sss_fp64_mma_peak, mma.sync "
                                                 "m8n8k4 f64); below the DFMA peak, so the "
                                                 "sparse vector action stays on DFMA"},
                         "flops_per_traj_step": fl},
            "clocks": clock_info,
            "fluorescence_check": float(np.mean(fluor))}
    if args.workload != "odmr":
        line["metric"] = {"ramsey": "NV-7 Ramsey (uneven) traj-steps/s",
                          "nv21": "NV-21 ODMR traj-steps/s"}[args.workload]
    if rank == 0 and world == 1 and args.workload == "odmr" and not args.rotating and \
            args.n_freq == N_FREQ and args.duration == DURATION:
        line["parity"] = full_length_parity(plan, N)
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.workload == "odmr" \
            and not args.rotating:
        cb = cpu_baseline(n_freq=args.n_freq)
        cb.pop("seconds", None)
        ref = cb.pop("states")
        line["cpu_baseline"] = cb
        line["cpu_algorithm_matched"] = cpu_vector_baseline(n_freq=args.n_freq)
        # the same trajectory and window through the batched path, against
        # the reference algorithm's states of the CPU baseline run
        ro_p, _, tr_p = plan.batch(rho0[:1], progs[:1], 0.0, DT_OUT, CPU_SAMPLES, F,
                                   readout_weights=w, want_trace=True)
        fl_ref = ref @ w
        line["parity_cpu_window"] = {
            "vs": "the reference's algorithm (CPU oracle, reference mode) run live on "
                  f"trajectory 0, {CPU_SAMPLES} samples x F={F}",
            "density_max_abs": float(np.abs(tr_p[0] - ref).max()),
            "fluorescence_rel_max": float(np.abs(ro_p[0] - fl_ref).max()/np.abs(fl_ref).max())}
    if rank == 0 and world == 1 and args.workload == "odmr" and not args.rotating and \
            not args.no_adjoint:
        line["adjoint"] = adjoint_measurement()
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
