"""CPU oracle for the time-stepping hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` import this module: to check the CUDA path's results, or as
the timed CPU baseline.  The product package never imports it.

It wraps ``sss_oracle.c`` (built by ``oracle/Makefile`` into
``oracle/_build/libsss_oracle.so``) and restates in numpy the host-side
parts of the reference's ``simulate`` (monashNV/superspinsim 1.3.2,
``superspinsim/generate_simulator.py``):

* the sample count ``int((tf - t0)/dt)`` (:1519);
* flattening rho0 through the vectorisation map (:1524-1549) and the
  unflattening with the Hermitian mirror (:2156-2191);
* the generalised rotating frame's host preparation (:1567-1677): the
  residual-aware e^{L0 h} blocks and the per-node rotating generators.

The quadrature tables are inputs here (the tests pass the reference's own
tables, stored in ``tests/golden/quadratures.npz``).

Parity pinned: the fixtures in ``tests/golden`` hold outputs of the
reference itself on the same inputs.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsss_oracle.so")

_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < os.path.getmtime(
                os.path.join(HERE, "sss_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        i = ctypes.c_int
        d = ctypes.c_double
        L.sss_oracle_simulate.argtypes = [
            i, i, i, i, dp, dp, dp, i, dp, i, dp, i, dp, dp, i, i, i, dp, i,
            i, d, d, i, i, i, dp, dp, i, i]
        L.sss_oracle_simulate.restype = i
        L.sss_oracle_max_threads.restype = i
        _lib = L
    return _lib


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def number_of_samples(t0, tf, dt):
    """generate_simulator.py:1519 -- truncating division."""
    return int((tf - t0)/dt)


def flatten(rho, vmap, N):
    """(n, n) complex -> (N,) real, generate_simulator.py:1524-1549."""
    n = rho.shape[0]
    real = np.empty((n, n, 2))
    real[:, :, 0] = np.real(rho)
    real[:, :, 1] = np.imag(rho)
    flat = np.empty(N)
    for i in range(N):
        if vmap is not None:
            y, x, c = vmap[i]
        else:
            h = int(math.sqrt(N//2))
            c, x, y = i % 2, (i//2) % h, (i//2)//h
        flat[i] = real[y, x, c]
    return flat


def unflatten(flat, vmap, n):
    """(..., N) real -> (..., n, n) complex, generate_simulator.py:2156-2191."""
    N = flat.shape[-1]
    out = np.zeros(flat.shape[:-1] + (n, n, 2))
    for i in range(N):
        if vmap is not None:
            y, x, c = vmap[i]
        else:
            h = int(math.sqrt(N//2))
            c, x, y = i % 2, (i//2) % h, (i//2)//h
        out[..., y, x, c] = flat[..., i]
        if vmap is not None and y != x:
            out[..., x, y, c] = -flat[..., i] if c else flat[..., i]
    return out[..., 0] + 1j*out[..., 1]


def rotating_tables(generators_rotating, doubles, singles, nodes, dt, F,
                    residual):
    """Host preparation of the rotating frame, generate_simulator.py:
    1567-1677.  Returns (gens (Q, G, N, N), doubles_last (D, 2),
    singles_last (S,))."""
    Q = nodes.size
    gens = np.asarray(generators_rotating, dtype=np.float64)
    doubles = np.asarray(doubles, dtype=np.float64).reshape(-1, 2)
    singles = np.asarray(singles, dtype=np.float64)
    tz = np.empty(Q + 1)
    tz[:-1] = nodes*dt/F
    tz[-1] = dt/F
    sf = np.empty((Q + 1, singles.size))
    sb = np.empty_like(sf)
    for i in range(Q + 1 - int(residual)):
        sf[i] = np.exp(singles*tz[i])
        sb[i] = np.exp(-singles*tz[i])
    df = np.empty((Q + 1, doubles.shape[0], 2))
    db = np.empty_like(df)
    for i in range(Q + 1 - int(residual)):
        att = np.exp(doubles[:, 0]*tz[i])
        amp = np.exp(-doubles[:, 0]*tz[i])
        s = np.sin(doubles[:, 1]*tz[i])
        c = np.cos(doubles[:, 1]*tz[i])
        df[i, :, 0] = att*c
        df[i, :, 1] = -att*s
        db[i, :, 0] = amp*c
        db[i, :, 1] = amp*s
    if residual:
        sf[-1] = np.expm1(singles*tz[-1])
        sin2 = -2*(np.sin(doubles[:, 1]*tz[-1]/2)**2)
        sin1 = np.sin(doubles[:, 1]*tz[-1])
        expmr = np.expm1(doubles[:, 0]*tz[-1])
        df[-1, :, 0] = (1 + expmr)*sin2 + expmr
        df[-1, :, 1] = -(1 + expmr)*sin1
    D = doubles.shape[0]
    out = np.empty((Q,) + gens.shape)
    for k in range(Q):
        g = gens.copy()
        for e in range(D):
            re = db[k, e, 0]*g[:, 2*e, :] - db[k, e, 1]*g[:, 2*e + 1, :]
            im = db[k, e, 1]*g[:, 2*e, :] + db[k, e, 0]*g[:, 2*e + 1, :]
            g[:, 2*e, :] = re
            g[:, 2*e + 1, :] = im
        for e in range(singles.shape[0]):
            g[:, 2*D + e, :] *= sb[k, e]
        for e in range(D):
            re = df[k, e, 0]*g[:, :, 2*e] + df[k, e, 1]*g[:, :, 2*e + 1]
            im = df[k, e, 1]*g[:, :, 2*e] - df[k, e, 0]*g[:, :, 2*e + 1]
            g[:, :, 2*e] = re
            g[:, :, 2*e + 1] = -im
        for e in range(singles.shape[0]):
            g[:, :, 2*D + e] *= sf[k, e]
        out[k] = g
    return out, np.ascontiguousarray(df[-1]), np.ascontiguousarray(sf[-1])


def simulate_flat(generators, flat0, t0, tf, dt, programs, *, K, W, nodes, F,
                  R=35, residual=True, rotating=None, mode="reference", degree=12,
                  threads=0):
    """The oracle on flattened states: flat0 (B, N) in the lab basis,
    programs (B, 4, S, 5).  Returns (time (T,), states (B, T, N)), lab
    basis."""
    W = np.ascontiguousarray(W, dtype=np.float64)
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    Kw, Q = W.shape
    assert Kw == K
    flat0 = np.asarray(flat0, dtype=np.float64)
    programs = np.asarray(programs, dtype=np.float64)
    B = flat0.shape[0]
    T = number_of_samples(t0, tf, dt)
    if rotating is not None:
        gens, dlast, slast = rotating_tables(
            rotating["generators_rotating"], rotating["doubles"],
            rotating["singles"], nodes, dt, F, residual)
        V = np.ascontiguousarray(rotating["vectors_real"], dtype=np.float64)
        Vi = np.ascontiguousarray(rotating["inv_vectors_real"],
                                  dtype=np.float64)
        D, S = dlast.shape[0], slast.size
        G = gens.shape[1]
        N = gens.shape[2]
    else:
        gens = np.asarray(generators, dtype=np.float64)
        G, N = gens.shape[0], gens.shape[1]
        dlast = slast = V = Vi = None
        D = S = 0
    gens = np.ascontiguousarray(gens)
    if rotating is not None and mode == "vector":
        flat0 = flat0 @ Vi.T
    flat0 = np.ascontiguousarray(flat0)
    progs = np.ascontiguousarray(programs)
    nch, nseg = progs.shape[1], progs.shape[2]
    out = np.zeros((B, T, N))
    status = lib().sss_oracle_simulate(
        N, G, K, Q, _ptr(gens), _ptr(W), _ptr(nodes), int(rotating is not None),
        _ptr(dlast), D, _ptr(slast), S, _ptr(V), _ptr(Vi), int(residual),
        int(R), int(degree), _ptr(progs), nch, nseg, float(t0), float(dt), T,
        int(F), B, _ptr(flat0), _ptr(out),
        0 if mode == "reference" else 1, int(threads))
    if status != 0:
        raise RuntimeError(f"oracle failed with status {status}")
    if rotating is not None and mode == "vector":
        out = out @ V.T
    return t0 + dt*(np.arange(T) + 1), out


def simulate(generators, rho0, t0, tf, dt, programs, *, K, W, nodes, F,
             R=35, residual=True, vectorisation_map=None, rotating=None,
             mode="reference", degree=12, threads=0, flat_out=False):
    """Run the oracle for one or more trajectories.

    generators: (G, N, N) lab-frame generators (when ``rotating`` is given,
        the rotating-frame generators from ``make_rotating`` go in
        ``rotating["generators_rotating"]`` and this argument is unused).
    rho0: (n, n) complex, or (B, n, n) for B trajectories.
    programs: (4, S, 5) coefficient program, or (B, 4, S, 5).
    rotating: dict with generators_rotating, vectors_real,
        inv_vectors_real, doubles, singles (reference make_rotating output).
    mode: "reference" (the reference's algorithm) or "vector".
    Returns (time (T,), density (T, n, n) or (B, T, n, n) complex).
    """
    single = np.asarray(rho0).ndim == 2
    rho0 = np.asarray(rho0)
    programs = np.asarray(programs, dtype=np.float64)
    if single:
        rho0 = rho0[None]
        programs = programs[None]
    n = rho0.shape[1]
    if rotating is not None:
        N = np.asarray(rotating["generators_rotating"]).shape[-1]
    else:
        N = np.asarray(generators).shape[1]
    flat0 = np.stack([flatten(r, vectorisation_map, N) for r in rho0])
    time, out = simulate_flat(generators, flat0, t0, tf, dt, programs, K=K, W=W,
                              nodes=nodes, F=F, R=R, residual=residual,
                              rotating=rotating, mode=mode, degree=degree,
                              threads=threads)
    res = out if flat_out else unflatten(out, vectorisation_map, n)
    return time, (res[0] if single else res)


def simulate_kernel(generators_image, image_projection, rho0, t0, tf, dt,
                    programs, *, vectorisation_map, rotating=None, **kw):
    """Equivalence-class mode as the reference intends it
    (generate_simulator.py:2043-2071): the generators act on the image of P
    (n_full x r) and the common-kernel components stay fixed, rho(t) = rho0 +
    P (U_r(t) - I) P^T rho0.  rho0 (n, n); returns (time, density (T, n, n))."""
    P = np.asarray(image_projection, dtype=np.float64)
    flat = flatten(np.asarray(rho0), vectorisation_map, P.shape[0])
    x0 = P.T @ flat
    time, out = simulate_flat(generators_image, x0[None], t0, tf, dt,
                              np.asarray(programs)[None], rotating=rotating, **kw)
    full = flat[None] + (out[0] - x0[None]) @ P.T
    return time, unflatten(full, vectorisation_map, np.asarray(rho0).shape[0])


def simulate_unitary(generators, rho0, t0, tf, dt, programs, *,
                     vectorisation_map, rotating=None, **kw):
    """Unitary mode as the reference's pipeline intends it
    (generate_simulator.py:2074-2101, Kronecker product :1394-1425): the
    real 2n x 2n generators propagate the operator U column by column, and
    the density is conj(U) rho0 U^T.  rho0 (n, n); returns (time, density
    (T, n, n)); ``vectorisation_map`` is not needed (full matrices)."""
    rho0 = np.asarray(rho0, dtype=complex)
    n = rho0.shape[0]
    cols = np.zeros((n, 2*n))
    for j in range(n):
        cols[j, 2*j] = 1.0
    progs = np.repeat(np.asarray(programs)[None], n, axis=0)
    time, out = simulate_flat(generators, cols, t0, tf, dt, progs, rotating=rotating, **kw)
    U = np.transpose(out[:, :, 0::2] + 1j*out[:, :, 1::2], (1, 2, 0))  # (T, n, n)
    return time, np.conj(U) @ rho0 @ np.transpose(U, (0, 2, 1))


def max_threads():
    return lib().sss_oracle_max_threads()
