"""Generalised rotating frame: real block diagonalisation of L0.

Restates ``_real_eig`` / ``make_rotating`` of the reference
(superspinsim/generate_generators.py:2390-2519): the eigenvectors of the
quiescent generator L0 are turned into a real basis -- a complex pair
contributes its real and imaginary parts (a 2x2 rotation-decay block,
"double"), a real eigenvalue its real vector ("single") -- keeping a vector
only when it raises the rank of the basis collected so far.  Doubles are
ordered by decreasing |lambda|, singles by decreasing |lambda|; the basis
is doubles (re, im pairs) then singles.  The time-dependent generators are
then expressed in that basis, G' = V^-1 G V.
"""
import math

import numpy as np

RANK_RTOL = 1e-16


class RotatingFrameError(Exception):
    """L0's eigenvectors do not span the space (the basis is singular)."""


def _rank(vectors):
    a = np.array(vectors).T
    s = np.linalg.svd(a, compute_uv=False)
    if s.size == 0 or s.max() == 0:
        return 0
    return int(np.sum(s > RANK_RTOL*s.max()))


def real_eig(generator):
    """(V, V^-1, doubles (D, 2) = (re, im), singles (S,))."""
    values, vectors = np.linalg.eig(generator)
    basis, best = [], 0
    doubles, singles = [], []
    for i in range(vectors.shape[1]):
        re = np.real(vectors[:, i]).copy()
        rank = _rank(basis + [re])
        if rank <= best:
            continue
        best = rank
        re /= math.sqrt(np.sum(re**2))
        basis.append(re)
        im = np.imag(vectors[:, i]).copy()
        rank = _rank(basis + [im])
        if rank > best:
            best = rank
            im /= math.sqrt(np.sum(im**2))
            basis.append(im)
            doubles.append(((np.real(values[i]), np.imag(values[i])), (re, im)))
        else:
            singles.append((np.real(values[i]), re))
    doubles.sort(key=lambda x: -(x[0][0]**2 + x[0][1]**2))
    singles.sort(key=lambda x: -abs(x[0]))
    cols = [v for _, pair in doubles for v in pair] + [v for _, v in singles]
    V = np.array(cols).T
    try:
        Vinv = np.linalg.inv(V)
    except np.linalg.LinAlgError as e:
        raise RotatingFrameError from e
    d = np.array([val for val, _ in doubles]).reshape(-1, 2)
    s = np.array([val for val, _ in singles])
    return V, Vinv, d, s


def make_rotating(superoperator_quiescent, superoperators_time_dependent):
    """(generators in the eigenbasis, V, V^-1, doubles, singles)."""
    V, Vinv, d, s = real_eig(superoperator_quiescent)
    gens = [Vinv @ g @ V for g in superoperators_time_dependent]
    return gens, V, Vinv, d, s
