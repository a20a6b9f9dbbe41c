"""Drop-in ``generate_simulator`` on the GB300 CUDA core.

Same signature and return convention as the reference's
``superspinsim/generate_simulator.py:17-47`` (``generate_simulator``) and
``:1508-2200`` (``simulate``): the returned ``simulate(rho0, t0, tf, dt)``
gives ``(time (T,), density (T, n, n) complex128)`` with
``T = int((tf - t0)/dt)`` output samples at ``t0 + dt*(t+1)``
(:1519, :158-159), each integrated with ``number_of_fine_divisions``
commutator-free Magnus steps.

The device work runs in libsss.so (include/sss.h) through ctypes.  The host
side here does what the reference's host side does: flattening rho0 through
the vectorisation map (:1524-1549), the generalised rotating frame's table
preparation (:1567-1677), and unflattening with the Hermitian mirror
(:2156-2191).

Coefficients: ``sampler`` is either a ``superspinsim_gb300.program.Program``
(evaluated on the GPU) or, as in the reference, a callable
``sampler(time, row)`` writing the G coefficients; a callable is sampled on
the host at every node time into a table that is uploaded with the run.

Equivalence-class mode (``use_kernel`` with ``image_projection`` P): the
generators act on the image of P and the states keep their full size; the
device lifts the result, rho(t) = rho0 + P (U_r - I) P^T rho0 (the form the
reference's sandwich and kernel addition intend, :1789-1797, :2043-2071).
Unitary mode (``use_unitary``): the generators are real 2n x 2n operator
forms and the device returns conj(U) rho0 U^T, what the reference's
Kronecker product and elimination/duplication sandwich give (:2074-2101);
the elimination and duplication matrices are accepted but not needed.

Differences from the reference, all raising instead of silently changing
behaviour: ``use_cuda=False`` (there is no CPU path), a ``datatype`` other
than float64, kernel and unitary modes together, and either mode beyond the
dense path's size; ``use_cayley`` raises ``TypeError`` as the reference's
``raise "..."`` does (:53-54).

``expm`` selects the exponential: ``"taylor"`` (default; degree-12 Taylor
polynomial after norm-chosen scaling, accurate to rounding) or
``"reference"`` (the reference's first-order Taylor after 4^-R scaling
followed by 2R squarings, in its operation order).
"""
import math

import numpy as np

from superspinsim_gb300 import _lib
from superspinsim_gb300.program import Program
from superspinsim_gb300.quadratures import method


PLAIN_MAX_N = 52   # dense shared-memory propagator path (csrc/sss_plain.cu)


def number_of_samples(time_start, time_end, time_step):
    return int((time_end - time_start)/time_step)


def _index_triples(N, vectorisation_map):
    if vectorisation_map is not None:
        vm = np.asarray(vectorisation_map)
        return vm[:, 0], vm[:, 1], vm[:, 2]
    n = int(math.sqrt(N//2))
    i = np.arange(N)
    return (i//2)//n, (i//2) % n, i % 2


def flatten_density(rho, N, vectorisation_map):
    """(..., n, n) complex -> (..., N) real in the reference's basis."""
    rho = np.asarray(rho)
    y, x, c = _index_triples(N, vectorisation_map)
    parts = np.stack([np.real(rho), np.imag(rho)], axis=-1)
    return np.ascontiguousarray(parts[..., y, x, c], dtype=np.float64)


def unflatten_density(flat, n, vectorisation_map):
    """(..., N) real -> (..., n, n) complex, mirroring Hermitian pairs."""
    flat = np.asarray(flat)
    N = flat.shape[-1]
    y, x, c = _index_triples(N, vectorisation_map)
    out = np.zeros(flat.shape[:-1] + (n, n, 2))
    out[..., y, x, c] = flat
    if vectorisation_map is not None:
        off = y != x
        sign = np.where(c[off] == 1, -1.0, 1.0)
        out[..., x[off], y[off], c[off]] = flat[..., off]*sign
    return out[..., 0] + 1j*out[..., 1]


def rotating_tables(generators, doubles, singles, nodes, fine_step, residual):
    """Per-node rotating generators and the one-step e^{L0 h} blocks.

    generators: (G, N, N) in the eigenbasis of L0 (make_rotating output);
    doubles (D, 2) = (decay, frequency) of the 2x2 blocks, singles (S,).
    Node k's generators are e^{-L0 tau_k} G e^{L0 tau_k} with
    tau_k = node_k*h, and the step table is e^{L0 h} (minus the identity
    in residual form, with expm1 and the half-angle sine for accuracy).
    Mirrors superspinsim/generate_simulator.py:1567-1677.
    """
    gens = np.asarray(generators, dtype=np.float64)
    doubles = np.asarray(doubles, dtype=np.float64).reshape(-1, 2)
    singles = np.asarray(singles, dtype=np.float64).reshape(-1)
    D, S = doubles.shape[0], singles.size
    Q = len(nodes)
    out = np.empty((Q,) + gens.shape)
    for k in range(Q):
        tau = nodes[k]*fine_step
        g = gens.copy()
        # rows: e^{-L0 tau}
        a = np.exp(-doubles[:, 0]*tau)
        cs, sn = np.cos(doubles[:, 1]*tau), np.sin(doubles[:, 1]*tau)
        bc, bs = a*cs, a*sn
        for e in range(D):
            r0, r1 = g[:, 2*e, :].copy(), g[:, 2*e + 1, :].copy()
            g[:, 2*e, :] = bc[e]*r0 - bs[e]*r1
            g[:, 2*e + 1, :] = bs[e]*r0 + bc[e]*r1
        g[:, 2*D:, :] *= np.exp(-singles*tau)[None, :, None]
        # columns: e^{L0 tau}
        f = np.exp(doubles[:, 0]*tau)
        fc, fs = f*cs, -f*sn
        for e in range(D):
            c0, c1 = g[:, :, 2*e].copy(), g[:, :, 2*e + 1].copy()
            g[:, :, 2*e] = fc[e]*c0 + fs[e]*c1
            g[:, :, 2*e + 1] = -(fs[e]*c0 - fc[e]*c1)
        g[:, :, 2*D:] *= np.exp(singles*tau)[None, None, :]
        out[k] = g
    h = fine_step
    if residual:
        sl = np.expm1(singles*h)
        em = np.expm1(doubles[:, 0]*h)
        half = -2*np.sin(doubles[:, 1]*h/2)**2
        dl = np.stack([(1 + em)*half + em, -(1 + em)*np.sin(doubles[:, 1]*h)], axis=1)
    else:
        sl = np.exp(singles*h)
        f = np.exp(doubles[:, 0]*h)
        dl = np.stack([f*np.cos(doubles[:, 1]*h), -f*np.sin(doubles[:, 1]*h)], axis=1)
    return out, np.ascontiguousarray(dl), np.ascontiguousarray(sl)


def sample_table(sampler, G, t0, dt, T, F, nodes):
    """Host sampling of a callable sampler at every node time, in the
    reference's row order (fine step r, sample t, node k)."""
    Q = len(nodes)
    tab = np.zeros((F, T, Q, G))
    row = np.zeros(G)
    for r in range(F):
        start = t0 + r*dt/F
        for t in range(T):
            base = start + dt*t
            for k in range(Q):
                row[:] = 0.0
                sampler(base + dt*nodes[k]/F, row)
                tab[r, t, k] = row
    return tab.reshape(1, F*T*Q, G)


def generate_simulator(
        sampler, generators, vectorisation_map=None, use_cuda=True,
        datatype=np.float64, use_residual=True, number_of_quartic_repeats=35,
        number_of_exponentials=2, number_of_fine_divisions=1,
        use_rotating=False, vectors_real=None, inv_vectors_real=None,
        doubles=None, singles=None, use_kernel=False, full_projection=None,
        image_projection=None, use_unitary=False, elimination=None,
        duplication=None, use_hermitian=True, verbose=False,
        use_cayley=False, expm="taylor"):
    """Build ``simulate(rho0, t0, tf, dt)`` for the given generators."""
    if not use_cuda:
        raise NotImplementedError("superspinsim_gb300 runs on the GPU only")
    if np.dtype(datatype) != np.float64:
        raise NotImplementedError("only float64 is supported")
    if use_cayley:
        raise TypeError("Cayley not implemented")
    if use_kernel and use_unitary:
        raise NotImplementedError("kernel and unitary modes together are not supported")
    if expm not in ("taylor", "reference"):
        raise ValueError("expm must be 'taylor' or 'reference'")
    generators = np.ascontiguousarray(generators, dtype=np.float64)
    G, N, _ = generators.shape
    if use_hermitian and vectorisation_map is None:
        use_hermitian = False
    vmap = np.asarray(vectorisation_map) if use_hermitian else None
    projection = None
    if use_kernel:
        if image_projection is None:
            raise ValueError("use_kernel needs image_projection")
        projection = np.ascontiguousarray(image_projection, dtype=np.float64)
        if projection.ndim != 2 or projection.shape[1] != N:
            raise ValueError("image_projection must be (full size, generator size)")
        Ns = projection.shape[0]          # entries of a flattened density
    elif use_unitary:
        if N % 2:
            raise ValueError("unitary generators must have an even size (2n)")
        Ns = vmap.shape[0] if vmap is not None else 2*(N//2)**2
    else:
        Ns = N
    if vmap is not None and vmap.shape[0] != Ns:
        raise ValueError("vectorisation_map rows must equal the state size")
    W, nodes = method(number_of_exponentials)
    F = int(number_of_fine_divisions)
    expm_code = _lib.SSS_EXPM_TAYLOR if expm == "taylor" else _lib.SSS_EXPM_REFERENCE
    state = {"plan": None, "h": None}

    def with_mode(plan):
        if projection is not None:
            plan.set_projection(projection)
        elif use_unitary:
            plan.set_unitary(N//2, vmap)
        return plan

    def plan_for(fine_step):
        if not use_rotating:
            if state["plan"] is None:
                state["plan"] = with_mode(_lib.Plan(generators, W, nodes, residual=use_residual,
                                                    expm=expm_code,
                                                    quartic_repeats=number_of_quartic_repeats))
            return state["plan"]
        if state["plan"] is None or state["h"] != fine_step:
            gn, dl, sl = rotating_tables(generators, doubles, singles, nodes, fine_step,
                                         use_residual)
            state["plan"] = _lib.Plan(None, W, nodes, residual=use_residual, expm=expm_code,
                                      quartic_repeats=number_of_quartic_repeats,
                                      rotating=dict(generators_nodes=gn, doubles_last=dl,
                                                    singles_last=sl,
                                                    vectors_real=vectors_real,
                                                    inv_vectors_real=inv_vectors_real))
            with_mode(state["plan"])
            state["h"] = fine_step
        return state["plan"]

    def simulate(density_operator_initial, time_start, time_end, time_step):
        T = number_of_samples(time_start, time_end, time_step)
        rho0 = np.asarray(density_operator_initial)
        n = rho0.shape[0]
        time = time_start + time_step*(np.arange(T) + 1)
        if T <= 0:
            return time, np.zeros((0, n, n), dtype=np.complex128)
        flat0 = flatten_density(rho0, Ns, vmap)[None]
        if N > PLAIN_MAX_N and (use_kernel or use_unitary):
            raise NotImplementedError(
                f"N = {N} > {PLAIN_MAX_N}: kernel and unitary modes run on the dense path only")
        if N > PLAIN_MAX_N:
            # larger than the dense shared-memory propagator path: the same
            # integrator through the batched kernel, full state per sample
            # (a callable sampler is sampled on the host into a coefficient
            # table, as for the dense path)
            if expm != "taylor":
                raise NotImplementedError(
                    f"N = {N} > {PLAIN_MAX_N}: only expm='taylor' is supported at this size")
            plan = plan_for(time_step/F)
            if isinstance(sampler, (Program, np.ndarray)):
                prog = sampler.as_array() if isinstance(sampler, Program) else sampler
                _, _, tr = plan.batch(flat0, prog[None], time_start, time_step, T, F,
                                      want_trace=True)
            else:
                tab = sample_table(sampler, G, time_start, time_step, T, F, nodes)
                _, _, tr = plan.batch(flat0, None, time_start, time_step, T, F,
                                      want_trace=True, table=tab)
            return time, unflatten_density(tr[0], n, vmap)
        plan = plan_for(time_step/F)
        if isinstance(sampler, Program):
            states = plan.simulate(flat0, sampler.as_array()[None], time_start, time_step, T, F)
        elif isinstance(sampler, np.ndarray) and sampler.ndim == 3 and sampler.shape[2] == 5:
            states = plan.simulate(flat0, sampler[None], time_start, time_step, T, F)
        else:
            tab = sample_table(sampler, G, time_start, time_step, T, F, nodes)
            states = plan.simulate(flat0, None, time_start, time_step, T, F, table=tab)
        return time, unflatten_density(states[0], n, vmap)

    return simulate
