"""Front end: ``simspins`` (reference superspinsim/sugar.py:385-584).

Builds the generators of a spin description, optionally moves to the
generalised rotating frame, and runs the GPU simulator.  Same arguments and
return value as the reference.  ``coefficients`` is either the reference's
list of four callables (x, y, z field in tesla, optical excitation) --
sampled on the host -- or a ``Program`` evaluated on the GPU.
"""
import numpy as np

from superspinsim_gb300.generate_simulator import generate_simulator
from superspinsim_gb300.generators import generate_atoms
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
    """Simulate a spin description; returns (time (T,), density (T, n, n))."""
    if use_kernel:
        raise NotImplementedError("equivalence-class (use_kernel) mode is not implemented")
    if use_unitary:
        raise NotImplementedError("unitary (use_unitary) mode is not implemented")
    ops, vmap = generate_atoms(spins, spin_interactions, group_interactions,
                               use_hermitian=use_hermitian, use_incoherent=use_incoherent)
    gens = [ops["generators"][k] for k in LABELS]
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
        use_hermitian=use_hermitian, verbose=verbose, expm=expm, **rotating)
    return sim(density_initial, time_start, time_end, time_step)
