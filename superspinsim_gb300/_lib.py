"""ctypes binding of libsss.so (include/sss.h).

The library is the only compute path of this package: if it is missing or
cannot be loaded, or no CUDA device is present, calls fail loudly -- there
is no CPU fallback.
"""
import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsss.so")

SSS_RESIDUAL = 1
SSS_ROTATING = 2
SSS_EXPM_REFERENCE = 0
SSS_EXPM_TAYLOR = 1

ERRORS = {-1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "ETIMEOUT",
          -5: "ENONFINITE", -6: "ENODEVICE"}

SYMBOLS = ["sss_plan_create", "sss_plan_set_rotating", "sss_simulate",
           "sss_simulate_device", "sss_batch_run", "sss_batch_run_table", "sss_plan_last_launches",
           "sss_plan_set_batch_config", "sss_plan_batch_info", "sss_plan_set_adjoint_memory",
           "sss_plan_set_projection", "sss_plan_set_unitary",
           "sss_fp64_peak", "sss_fp64_mma_peak", "sss_simulate_noalloc", "sss_adjoint_run", "sss_adjoint_run_channel", "sss_batch_prepare",
           "sss_batch_prepare_samples", "sss_batch_launch", "sss_batch_check", "sss_slot_layout", "sss_plan_batch_work", "sss_plan_bank_conflicts", "sss_last_error",
           "sss_plan_destroy"]


class SSSError(RuntimeError):
    """An error code returned by libsss.so."""

    def __init__(self, code, message):
        super().__init__(f"libsss {ERRORS.get(code, code)}: {message}")
        self.code = code


class PlanDesc(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("G", ctypes.c_int), ("K", ctypes.c_int),
                ("Q", ctypes.c_int), ("flags", ctypes.c_uint),
                ("expm", ctypes.c_int), ("quartic_repeats", ctypes.c_int),
                ("taylor_degree", ctypes.c_int)]


_lib = None
_lock = threading.Lock()


def load(build_if_missing=True):
    """Load libsss.so (building it in-tree with nvcc if it is absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise RuntimeError(f"{LIB_PATH} is missing; run "
                                   "superspinsim_gb300.build.build()")
            from superspinsim_gb300 import build
            build.build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        vp = ctypes.c_void_p
        i, d = ctypes.c_int, ctypes.c_double
        L.sss_plan_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(PlanDesc),
                                      dp, dp, dp]
        L.sss_plan_set_rotating.argtypes = [vp, dp, dp, i, dp, i, dp, dp]
        sim = [vp, i, dp, i, i, dp, dp, d, d, i, i, dp, vp]
        L.sss_simulate.argtypes = sim
        L.sss_simulate_device.argtypes = [vp, i, vp, i, i, vp, vp, d, d, i, i, vp, vp]
        L.sss_batch_run.argtypes = [vp, i, vp, i, i, vp, vp, d, d, i, i, dp, vp, vp, vp, i, vp]
        L.sss_batch_run_table.argtypes = [vp, i, vp, vp, vp, d, d, i, i, dp, vp, vp, vp, i, vp]
        L.sss_plan_last_launches.argtypes = [vp]
        L.sss_plan_set_batch_config.argtypes = [vp, i, i, i]
        L.sss_plan_set_adjoint_memory.argtypes = [vp, ctypes.c_size_t]
        L.sss_plan_set_adjoint_memory.restype = i
        L.sss_plan_set_projection.argtypes = [vp, i, dp]
        L.sss_plan_set_projection.restype = i
        L.sss_plan_set_unitary.argtypes = [vp, i, i, ctypes.POINTER(ctypes.c_int)]
        L.sss_plan_set_unitary.restype = i
        L.sss_plan_batch_info.argtypes = [vp, ip, ip, ip, ip, ip, dp]
        L.sss_fp64_peak.argtypes = [dp, vp]
        L.sss_fp64_mma_peak.argtypes = [dp, vp]
        L.sss_fp64_mma_peak.restype = i
        L.sss_adjoint_run.argtypes = [vp, i, vp, i, i, vp, d, d, i, i, dp, dp, vp, vp, i, vp]
        L.sss_adjoint_run.restype = i
        L.sss_adjoint_run_channel.argtypes = [vp, i, vp, i, i, vp, d, d, i, i, dp, dp, i, vp, vp,
                                              i, vp]
        L.sss_adjoint_run_channel.restype = i
        L.sss_batch_prepare.argtypes = [vp, i, vp, i, i, vp, d, i, dp, vp]
        L.sss_batch_prepare.restype = i
        L.sss_batch_prepare_samples.argtypes = [vp, i, vp, i, i, vp, vp, d, i, dp, vp]
        L.sss_batch_prepare_samples.restype = i
        L.sss_batch_launch.argtypes = [vp, vp, vp, vp, d, i, i, i, vp, vp]
        L.sss_batch_launch.restype = i
        L.sss_batch_check.argtypes = [vp, vp]
        L.sss_batch_check.restype = i
        L.sss_fp64_peak.restype = i
        L.sss_slot_layout.argtypes = [i, ip, ip, i, i, ip, ip, ip,
                                      ctypes.POINTER(ctypes.c_uint), ip]
        L.sss_slot_layout.restype = i
        L.sss_plan_batch_work.argtypes = [vp, ip, ip, ip, ip]
        L.sss_plan_batch_work.restype = i
        L.sss_plan_bank_conflicts.argtypes = [vp, ip, ip]
        L.sss_plan_bank_conflicts.restype = i
        L.sss_last_error.restype = ctypes.c_char_p
        L.sss_plan_destroy.argtypes = [vp]
        L.sss_plan_destroy.restype = None
        for name in ["sss_plan_create", "sss_plan_set_rotating", "sss_simulate",
                     "sss_simulate_device", "sss_batch_run",
                     "sss_plan_last_launches", "sss_plan_set_batch_config",
                     "sss_plan_batch_info"]:
            getattr(L, name).restype = i
        _lib = L
        return L


def check(code):
    if code != 0:
        msg = load().sss_last_error().decode(errors="replace")
        raise SSSError(code, msg)


def dptr(a):
    """Pointer to a C-contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


class Plan:
    """Owner of one sss_plan (device copies of generators and tables)."""

    def __init__(self, generators, weights, nodes, *, residual=True,
                 expm=SSS_EXPM_TAYLOR, quartic_repeats=35, taylor_degree=0,
                 rotating=None):
        L = load()
        weights = np.ascontiguousarray(weights, dtype=np.float64)
        nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        K, Q = weights.shape
        flags = SSS_RESIDUAL if residual else 0
        if rotating is not None:
            flags |= SSS_ROTATING
            gn = np.ascontiguousarray(rotating["generators_nodes"], dtype=np.float64)
            Qg, G, N, _ = gn.shape
            assert Qg == Q
            gens = None
        else:
            gens = np.ascontiguousarray(generators, dtype=np.float64)
            G, N, _ = gens.shape
        self.N, self.G, self.K, self.Q = N, G, K, Q
        self.n_state = N   # entries of a state in and of a sample out of simulate
        desc = PlanDesc(N, G, K, Q, flags, expm, quartic_repeats, taylor_degree)
        h = ctypes.c_void_p()
        check(L.sss_plan_create(ctypes.byref(h), ctypes.byref(desc), dptr(gens),
                                dptr(weights), dptr(nodes)))
        self._h = h
        if rotating is not None:
            dl = np.ascontiguousarray(rotating["doubles_last"], dtype=np.float64).reshape(-1, 2)
            sl = np.ascontiguousarray(rotating["singles_last"], dtype=np.float64)
            V = np.ascontiguousarray(rotating["vectors_real"], dtype=np.float64)
            Vi = np.ascontiguousarray(rotating["inv_vectors_real"], dtype=np.float64)
            check(L.sss_plan_set_rotating(h, dptr(gn), dptr(dl), dl.shape[0], dptr(sl),
                                          sl.size, dptr(V), dptr(Vi)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.sss_plan_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def set_projection(self, image_projection):
        """Equivalence-class mode: generators act on the image of P
        (n_full x N); simulate then takes and returns n_full-entry states.
        None clears it."""
        if image_projection is None:
            check(load().sss_plan_set_projection(self._h, 0, None))
            self.n_state = self.N
            return
        P = np.ascontiguousarray(image_projection, dtype=np.float64)
        check(load().sss_plan_set_projection(self._h, P.shape[0], dptr(P)))
        self.n_state = P.shape[0]

    def set_unitary(self, n, vectorisation_map=None):
        """Unitary mode for an n-level system (N = 2n operator generators);
        simulate then takes and returns densities flattened by the map (or
        all 2n^2 entries row-major).  n = 0 clears it."""
        if not n:
            check(load().sss_plan_set_unitary(self._h, 0, 0, None))
            self.n_state = self.N
            return
        if vectorisation_map is None:
            check(load().sss_plan_set_unitary(self._h, int(n), 0, None))
            self.n_state = 2*n*n
            return
        vm = np.ascontiguousarray(vectorisation_map, dtype=np.int32).reshape(-1, 3)
        check(load().sss_plan_set_unitary(self._h, int(n), vm.shape[0],
                                          vm.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        self.n_state = vm.shape[0]

    def simulate(self, rho0, programs, t0, dt, T, F, table=None, stream=None):
        """rho0 (B, n_state); programs (B, nch, nseg, 5) or None with table
        (B, F*T*Q, G).  Returns (B, T, n_state) (n_state = N unless a
        projection or unitary mode is set)."""
        rho0 = np.ascontiguousarray(rho0, dtype=np.float64)
        B = rho0.shape[0]
        if rho0.shape[1] != self.n_state:
            raise ValueError(f"rho0 has {rho0.shape[1]} entries per state, the plan takes "
                             f"{self.n_state}")
        out = np.empty((B, T, self.n_state))
        if programs is not None:
            programs = np.ascontiguousarray(programs, dtype=np.float64)
            nch, nseg = programs.shape[1], programs.shape[2]
        else:
            nch = nseg = 0
        if table is not None:
            table = np.ascontiguousarray(table, dtype=np.float64)
        check(load().sss_simulate(self._h, B, dptr(rho0), nch, nseg, dptr(programs),
                                  dptr(table), float(t0), float(dt), int(T), int(F),
                                  dptr(out), stream))
        return out

    def batch(self, rho0, programs, t0, dt, T_max, F, samples=None,
              readout_weights=None, want_final=False, stream=None, want_trace=False,
              table=None):
        """Host-buffer batched run.  Returns (readout (B, T_max) or None,
        final (B, N) or None[, trace (B, T_max, N)]).  `table` (B, F*T_max*Q,
        G) -- sampled coefficients in sss_simulate's row order -- replaces
        the programs (then None)."""
        rho0 = np.ascontiguousarray(rho0, dtype=np.float64)
        B = rho0.shape[0]
        ro = np.empty((B, T_max)) if readout_weights is not None else None
        fin = np.empty((B, self.N)) if want_final else None
        tr = np.empty((B, T_max, self.N)) if want_trace else None
        rw = None if readout_weights is None else np.ascontiguousarray(
            readout_weights, dtype=np.float64)
        smp = None if samples is None else np.ascontiguousarray(samples, dtype=np.int32)
        outs = (None if ro is None else ro.ctypes.data_as(ctypes.c_void_p),
                None if fin is None else fin.ctypes.data_as(ctypes.c_void_p),
                None if tr is None else tr.ctypes.data_as(ctypes.c_void_p))
        if table is not None:
            table = np.ascontiguousarray(table, dtype=np.float64)
            if table.shape != (B, F*T_max*self.Q, self.G):
                raise ValueError(f"coefficient table of shape {table.shape}, expected "
                                 f"{(B, F*T_max*self.Q, self.G)}")
            check(load().sss_batch_run_table(
                self._h, B, rho0.ctypes.data_as(ctypes.c_void_p),
                table.ctypes.data_as(ctypes.c_void_p), iptr(smp), float(t0), float(dt),
                int(T_max), int(F), dptr(rw), *outs, 1, stream))
        else:
            programs = np.ascontiguousarray(programs, dtype=np.float64)
            nch, nseg = programs.shape[1], programs.shape[2]
            check(load().sss_batch_run(
                self._h, B, rho0.ctypes.data_as(ctypes.c_void_p), nch, nseg,
                programs.ctypes.data_as(ctypes.c_void_p), iptr(smp), float(t0), float(dt),
                int(T_max), int(F), dptr(rw), *outs, 1, stream))
        if want_trace:
            return ro, fin, tr
        return ro, fin

    def batch_device(self, rho0_ptr, B, programs_ptr, nch, nseg, t0, dt, T_max,
                     F, samples_ptr=None, readout_weights=None, readout_ptr=None,
                     final_ptr=None, stream=None):
        """Device-pointer batched run (pointers as integers)."""
        rw = None if readout_weights is None else np.ascontiguousarray(
            readout_weights, dtype=np.float64)
        check(load().sss_batch_run(self._h, B, rho0_ptr, nch, nseg, programs_ptr,
                                   samples_ptr, float(t0), float(dt), int(T_max),
                                   int(F), dptr(rw), readout_ptr, final_ptr, None, 0, stream))

    def adjoint(self, rho0, programs, t0, dt, T, F, readout_weights, time_weights, stream=None):
        """Host-buffer adjoint run.  Returns (J (B,), grad (B, nseg, 2))."""
        rho0 = np.ascontiguousarray(rho0, dtype=np.float64)
        programs = np.ascontiguousarray(programs, dtype=np.float64)
        B = rho0.shape[0]
        nch, nseg = programs.shape[1], programs.shape[2]
        J = np.empty(B)
        grad = np.empty((B, nseg, 2))
        rw = np.ascontiguousarray(readout_weights, dtype=np.float64)
        tw = np.ascontiguousarray(time_weights, dtype=np.float64)
        assert tw.size == T
        check(load().sss_adjoint_run(
            self._h, B, rho0.ctypes.data_as(ctypes.c_void_p), nch, nseg,
            programs.ctypes.data_as(ctypes.c_void_p), float(t0), float(dt), int(T), int(F),
            dptr(rw), dptr(tw), J.ctypes.data_as(ctypes.c_void_p),
            grad.ctypes.data_as(ctypes.c_void_p), 1, stream))
        return J, grad

    def adjoint_channel(self, rho0, programs, t0, dt, T, F, readout_weights, time_weights,
                        channel, stream=None):
        """Host-buffer adjoint run for the segments of one channel.  Returns
        (J (B,), grad (B, nseg, 4)): d/d (amplitude, phase, offset,
        frequency) of every segment of `channel`."""
        rho0 = np.ascontiguousarray(rho0, dtype=np.float64)
        programs = np.ascontiguousarray(programs, dtype=np.float64)
        B = rho0.shape[0]
        nch, nseg = programs.shape[1], programs.shape[2]
        J = np.empty(B)
        grad = np.empty((B, nseg, 4))
        rw = np.ascontiguousarray(readout_weights, dtype=np.float64)
        tw = np.ascontiguousarray(time_weights, dtype=np.float64)
        assert tw.size == T
        check(load().sss_adjoint_run_channel(
            self._h, B, rho0.ctypes.data_as(ctypes.c_void_p), nch, nseg,
            programs.ctypes.data_as(ctypes.c_void_p), float(t0), float(dt), int(T), int(F),
            dptr(rw), dptr(tw), int(channel), J.ctypes.data_as(ctypes.c_void_p),
            grad.ctypes.data_as(ctypes.c_void_p), 1, stream))
        return J, grad

    def batch_prepare(self, rho0_ptr, B, programs_ptr, nch, nseg, dt, F,
                      readout_weights=None, stream=None, samples=None):
        """Analyse a batch (device pointers) and upload the kernel tables.
        `samples` (host, B) -- the trajectories' output-sample counts, the
        same as every launch passes -- prepares the phases of an uneven
        batch (sss_batch_prepare_samples)."""
        rw = None if readout_weights is None else np.ascontiguousarray(
            readout_weights, dtype=np.float64)
        if samples is None:
            check(load().sss_batch_prepare(self._h, B, rho0_ptr, nch, nseg, programs_ptr,
                                           float(dt), int(F), dptr(rw), stream))
        else:
            smp = np.ascontiguousarray(samples, dtype=np.int32)
            check(load().sss_batch_prepare_samples(self._h, B, rho0_ptr, nch, nseg, programs_ptr,
                                                   smp.ctypes.data_as(ctypes.c_void_p), float(dt),
                                                   int(F), dptr(rw), stream))

    def batch_launch(self, state_ptr, programs_ptr, t0, t_begin, n_samples, T_max,
                     samples_ptr=None, readout_ptr=None, stream=None):
        """Run output samples [t_begin, t_begin + n_samples) in place on state."""
        check(load().sss_batch_launch(self._h, state_ptr, programs_ptr, samples_ptr, float(t0),
                                      int(t_begin), int(n_samples), int(T_max), readout_ptr,
                                      stream))

    def batch_check(self, stream=None):
        """Wait for the stream; raise SSSError (ENONFINITE) if a launch since
        the last prepare or check wrote a NaN or infinite value."""
        check(load().sss_batch_check(self._h, stream))

    def set_batch_config(self, lanes=0, cta_threads=0, variant=0):
        check(load().sss_plan_set_batch_config(self._h, int(lanes), int(cta_threads),
                                               int(variant)))

    def set_adjoint_memory(self, max_bytes=0):
        """Device memory the adjoint may use for stored forward states
        (0: half of the free memory)."""
        check(load().sss_plan_set_adjoint_memory(self._h, int(max_bytes)))

    def batch_info(self):
        vals = [ctypes.c_int() for _ in range(5)]
        ms = ctypes.c_double()
        check(load().sss_plan_batch_info(self._h, *[ctypes.byref(v) for v in vals],
                                         ctypes.byref(ms)))
        out = dict(zip(["lanes", "degree", "substeps", "rows", "nnz"],
                       [v.value for v in vals]))
        out["kernel_ms"] = ms.value
        work = [ctypes.c_int() for _ in range(4)]
        check(load().sss_plan_batch_work(self._h, *[ctypes.byref(v) for v in work]))
        out.update(zip(["variant", "live_generators", "live_nnz", "fp64_per_term"],
                       [v.value for v in work]))
        bank = [ctypes.c_int() for _ in range(2)]
        check(load().sss_plan_bank_conflicts(self._h, *[ctypes.byref(v) for v in bank]))
        out["bank_extra_wavefronts_per_term"] = {"lane_order": bank[0].value,
                                                 "renumbered": bank[1].value}
        return out

    def last_launches(self):
        return load().sss_plan_last_launches(self._h)


def fp64_peak_tflops(stream=None, repeats=5):
    """Measured FP64 FMA throughput of the current GPU (TFLOP/s): the best
    of `repeats` probes (a probe taken while the clocks are still ramping
    up reads low)."""
    best = 0.0
    for _ in range(repeats):
        v = ctypes.c_double()
        check(load().sss_fp64_peak(ctypes.byref(v), stream))
        best = max(best, v.value)
    return best


def fp64_mma_peak_tflops(stream=None, repeats=5):
    """Measured FP64 tensor-core (DMMA) throughput of the current GPU
    (TFLOP/s), best of `repeats` probes."""
    best = 0.0
    for _ in range(repeats):
        v = ctypes.c_double()
        check(load().sss_fp64_mma_peak(ctypes.byref(v), stream))
        best = max(best, v.value)
    return best


SLOTS_MAX = 16


def slot_layout(row_ptr, col, lanes, max_slots=SLOTS_MAX):
    """The slot-packed layout of a row pattern (sss_slot_layout; host only).
    Returns (slots, barrier_slot, partials, words (slots, lanes) uint32,
    entries (slots, lanes) int: index into col, -1 close/padding, -2
    partial add)."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
    col = np.ascontiguousarray(col, dtype=np.int32)
    M = row_ptr.size - 1
    words = np.zeros(SLOTS_MAX*lanes, dtype=np.uint32)
    entries = np.zeros(SLOTS_MAX*lanes, dtype=np.int32)
    S, bar, npart = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    ip = ctypes.POINTER(ctypes.c_int)
    check(load().sss_slot_layout(
        M, row_ptr.ctypes.data_as(ip), col.ctypes.data_as(ip), int(lanes), int(max_slots),
        ctypes.byref(S), ctypes.byref(bar), ctypes.byref(npart),
        words.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), entries.ctypes.data_as(ip)))
    n = S.value
    return (n, bar.value, npart.value, words.reshape(SLOTS_MAX, lanes)[:n].copy(),
            entries.reshape(SLOTS_MAX, lanes)[:n].copy())
