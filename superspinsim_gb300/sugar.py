"""Front end: ``simspins`` (reference superspinsim/sugar.py:385-584).

Builds the generators of a spin description, optionally moves to the
generalised rotating frame, and runs the GPU simulator.  Same arguments and
return value as the reference.  ``coefficients`` is either the reference's
list of four callables (x, y, z field in tesla, optical excitation) --
sampled on the host -- or a ``Program`` evaluated on the GPU.
"""
import numpy as np

from superspinsim_gb300.generate_simulator import generate_simulator
from superspinsim_gb300.generators import find_kernel, generate_atoms
from superspinsim_gb300.program import Program
from superspinsim_gb300.rotating import RotatingFrameError, make_rotating

LABELS = ("L0", "Gx", "Gy", "Gz", "Gr")


def make_sampler(coefficients, use_rotating):
    """The coefficient row writer of the reference's front end
    (generate_generators.py:2317-2358): lab frame [1, x, y, z, r], rotating
    frame [x, y, z, r]."""
    if isinstance(coefficients, Program):
        return coefficients
    fx, fy, fz, fr = coefficients
    if use_rotating:
        def sampler(time, row):
            row[0] = fx(time)
            row[1] = fy(time)
            row[2] = fz(time)
            row[3] = fr(time)
    else:
        def sampler(time, row):
            row[0] = 1.0
            row[1] = fx(time)
            row[2] = fy(time)
            row[3] = fz(time)
            row[4] = fr(time)
    return sampler


def simspins(coefficients, time_start, time_end, time_step, spins, spin_interactions,
             group_interactions, density_initial, number_of_exponentials=5,
             number_of_fine_divisions=1, number_of_quadratic_repeats=35, use_rotating=True,
             use_residual=True, use_kernel=False, use_unitary=False, use_cuda=True,
             use_hermitian=True, use_incoherent=True, datatype=np.float64, verbose=False,
             expm="taylor"):
    """Simulate a spin description; returns (time (T,), density (T, n, n)).

    As the reference (sugar.py:472-534): ``use_unitary`` takes the operator
    generators when the system has no jump operators (else the Liouvillian
    ones), ``use_kernel`` restricts the generators to the complement of
    their common kernel, and the rotating frame is built on what results."""
    ops, vmap = generate_atoms(spins, spin_interactions, group_interactions,
                               use_unitary=use_unitary, use_hermitian=use_hermitian,
                               use_incoherent=use_incoherent)
    if use_unitary and "unitary" not in ops:
        use_unitary = False
    unitary = {}
    if use_unitary:
        gens = [ops["unitary"][k] for k in ("H0", "Gx", "Gy", "Gz", "Gr")]
        unitary = dict(ops["elimination"])
    else:
        gens = [ops["generators"][k] for k in LABELS]
    kernel = {}
    if use_kernel:
        full, image, gens_image = find_kernel(gens)
        if image.shape[1] == image.shape[0]:
            use_kernel = False      # no common kernel: nothing to remove
        elif use_unitary:
            raise NotImplementedError("kernel and unitary modes together are not supported")
        else:
            gens = gens_image
            kernel = dict(full_projection=full, image_projection=image)
    rotating = {}
    if use_rotating:
        if np.sum(np.abs(gens[0])) == 0:
            use_rotating = False
        else:
            try:
                new, V, Vinv, d, s = make_rotating(gens[0], gens[1:])
                gens = new
                rotating = dict(vectors_real=V, inv_vectors_real=Vinv, doubles=d, singles=s)
            except RotatingFrameError:
                print("Lindblad operator is not invertible.\nRotating frame cannot be used.")
                use_rotating = False
    sampler = make_sampler(coefficients, use_rotating)
    sim = generate_simulator(
        sampler, np.array(gens), vmap, use_cuda=use_cuda, datatype=datatype,
        use_residual=use_residual, number_of_quartic_repeats=number_of_quadratic_repeats,
        number_of_exponentials=number_of_exponentials,
        number_of_fine_divisions=number_of_fine_divisions, use_rotating=use_rotating,
        use_hermitian=use_hermitian, verbose=verbose, expm=expm, use_kernel=use_kernel,
        use_unitary=use_unitary, **rotating, **kernel, **unitary)
    return sim(density_initial, time_start, time_end, time_step)


def _sort_operators(operators, label):
    """Split an operator spec into (static list, time-dependent list,
    coefficient functions), as the reference's _sort_operators
    (superspinsim/sugar.py:164-212): an array; an [array, callable] pair; or
    a list of those.  Objects with a ``full()`` method (qutip.Qobj) are
    converted with it."""
    def as_array(o):
        if isinstance(o, np.ndarray):
            return o
        if hasattr(o, "full") and callable(o.full):
            return np.asarray(o.full())
        return None

    static, dynamic, coeffs = [], [], []
    if operators is None:
        return static, dynamic, coeffs
    a = as_array(operators)
    if a is not None:
        return [a], dynamic, coeffs
    if not isinstance(operators, list):
        raise TypeError(f"{label} must be numpy.ndarray, an [np.ndarray, function] list, "
                        "or list of either.")
    if len(operators) == 2 and as_array(operators[0]) is not None and callable(operators[1]):
        return static, [as_array(operators[0])], [operators[1]]
    for op in operators:
        a = as_array(op)
        if a is not None:
            static.append(a)
            continue
        if isinstance(op, (list, tuple)) and len(op) == 2 and as_array(op[0]) is not None \
                and callable(op[1]):
            dynamic.append(as_array(op[0]))
            coeffs.append(op[1])
            continue
        raise TypeError(f"{label} must be numpy.ndarray, an [np.ndarray, function] list, "
                        "or list of either.")
    return static, dynamic, coeffs


def mesolve(H, rho0, ti, tf, dt, c_ops=None, allowed=None, use_rotating=True,
            use_hermitian=True, number_of_exponentials=5, number_of_fine_divisions=10,
            use_cuda=True, expm="taylor"):
    """QuTiP-style front end (reference superspinsim/sugar.py:21-161):
    Hamiltonian and jump operators as arrays or [array, coefficient(t)]
    pairs; time-dependent jump coefficients enter through their square root,
    as in the reference.  Returns (time (T,), density (T, n, n))."""
    from superspinsim_gb300.generators import dissipator, valid_indices_from_mask, \
        von_neumann, _basis
    h_static, h_dyn, h_coef = _sort_operators(H, "H")
    l_static, l_dyn, l_coef = _sort_operators(c_ops, "c_ops")
    if not (h_static or h_dyn or l_static or l_dyn):
        raise TypeError("No operators specified.")
    n = (h_static + h_dyn + l_static + l_dyn)[0].shape[0]
    if allowed is None:
        allowed = np.ones((n, n))
    valid = valid_indices_from_mask(np.asarray(allowed))
    basis, sel = _basis(n, valid, use_hermitian)
    quiescent = None
    for Hs in ([sum(h_static)] if h_static else []):
        S = von_neumann(np.asarray(Hs, dtype=complex), basis, sel)
        quiescent = S if quiescent is None else quiescent + S
    for L in l_static:
        S = dissipator(np.asarray(L, dtype=complex), basis, sel)
        quiescent = S if quiescent is None else quiescent + S
    dynamic = [von_neumann(np.asarray(h, dtype=complex), basis, sel) for h in h_dyn]
    dynamic += [dissipator(np.asarray(L, dtype=complex), basis, sel) for L in l_dyn]
    if quiescent is None:
        quiescent = np.zeros_like(dynamic[0])
    coeffs = list(h_coef) + [(lambda f: (lambda t: np.sqrt(f(t))))(f) for f in l_coef]
    rotating = {}
    if use_rotating:
        try:
            dynamic, V, Vinv, d, s = make_rotating(quiescent, dynamic)
            rotating = dict(vectors_real=V, inv_vectors_real=Vinv, doubles=d, singles=s)
        except RotatingFrameError:
            print("Lindblad operator is not invertible.\nRotating frame cannot be used.")
            use_rotating = False
    gens = dynamic if use_rotating else [quiescent] + dynamic
    offset = 0 if use_rotating else 1

    def sampler(time, row):
        if not use_rotating:
            row[0] = 1.0
        for i, f in enumerate(coeffs):
            row[offset + i] = f(time)

    sim = generate_simulator(sampler, np.array(gens), valid if use_hermitian else None,
                             use_cuda=use_cuda, number_of_exponentials=number_of_exponentials,
                             number_of_fine_divisions=number_of_fine_divisions,
                             use_rotating=use_rotating, use_hermitian=use_hermitian, expm=expm,
                             **rotating)
    return sim(np.asarray(rho0), ti, tf, dt)
