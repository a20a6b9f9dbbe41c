"""Gauss-Legendre nodes and commutator-free Magnus weights.

Same tables, keys and layout as the reference's ``superspinsim/quadratures.py``
(:10-50, generated by ``superspinsim/generate_quadratures.py``), derived here
from the published construction:

* nodes c_k on [0, 1] of the 1-, 2- and 3-point Gauss-Legendre rules;
* weights rho = X R Q (Blanes & Moan, Appl. Numer. Math. 56 (2006) 1519,
  eq. 50): Q maps node samples to Legendre moments (their eq. 22), R
  rescales the moments (eq. 24), X holds the method coefficients (eq. 37
  for the 4th-order methods, Table 1 for the 6th-order ones, completed by
  the consistency conditions and the time-symmetry of eq. 33).

Row e of ``weights[key]`` gives the exponent of exponential e as a linear
combination of the generator samples at the nodes; in a step, exponential
K-1 acts first and exponential 0 last.
"""
import math

import numpy as np


def _gauss_legendre(q):
    x, _ = np.polynomial.legendre.leggauss(q)
    return np.sort((x + 1)/2)


def _moments(q):
    """Q: Legendre-moment quadrature matrix (rows: moments 0..q-1)."""
    if q == 1:
        return np.array([[1.0]])
    if q == 2:
        s = math.sqrt(3)/12
        return np.array([[0.5, 0.5], [-s, s]])
    s = math.sqrt(15)/36
    return np.array([[5/18, 4/9, 5/18], [-s, 0.0, s], [1/24, 0.0, 1/24]])


def _rescale(q):
    if q == 1:
        return np.array([[1.0]])
    if q == 2:
        return np.array([[1.0, 0.0], [0.0, 12.0]])
    return np.array([[9/4, 0.0, -15.0], [0.0, 12.0, 0.0], [-15.0, 0.0, 180.0]])


def _symmetric(top, rows):
    """Complete X by time symmetry: row K-1-e = (-1)^j * row e."""
    x = np.zeros((rows, top.shape[1]))
    x[:top.shape[0]] = top
    for e in range(rows//2):
        for j in range(x.shape[1]):
            x[rows - 1 - e, j] = (-1)**j*x[e, j]
    return x


def _method_coefficients():
    X = {"2_1_gl": np.array([[1.0]])}
    X["4_2_gl"] = _symmetric(np.array([[1/2, 1/6]]), 2)
    X["4_3_gl"] = _symmetric(np.array([[0.0, 1/12], [1.0, 0.0]]), 3)
    # CF6:5 and CF6:6, Blanes & Moan (2006) Table 1; the middle row follows
    # from sum_e x_e1 = 1 and sum_e x_e3 = 1/12 (CF6:5), resp. 1/2, 1/24
    # over the first half (CF6:6, whose middle rows pair up)
    x65 = np.array([[0.2, 0.08734395950888931101, 0.03734395950888931101],
                    [0.34815492558797391479, 0.053438272547684150,
                     0.00584269157837031012],
                    [0.0, 0.0, 0.0]])
    x65[2, 0] = 1 - 2*(x65[0, 0] + x65[1, 0])
    x65[2, 2] = 1/12 - 2*(x65[0, 2] + x65[1, 2])
    X["6_5_gl"] = _symmetric(x65, 5)
    x66 = np.array([[0.208, 0.09023186422416794596, 0.03823186422416794596],
                    [0.312, 0.04467385661651479788, 0.00439421553992544024],
                    [0.0, 0.01407960659498524468, 0.0]])
    x66[2, 0] = 1/2 - (x66[0, 0] + x66[1, 0])
    x66[2, 2] = 1/24 - (x66[0, 2] + x66[1, 2])
    X["6_6_gl"] = _symmetric(x66, 6)
    return X


_NODES_OF = {"2_1_gl": 1, "4_2_gl": 2, "4_3_gl": 2, "6_5_gl": 3, "6_6_gl": 3}

samples = {f"{q}_gl": _gauss_legendre(q) for q in (1, 2, 3)}
samples["1_gl"] = np.array([0.5])
samples["2_gl"] = np.array([0.5 - math.sqrt(3)/6, 0.5 + math.sqrt(3)/6])
samples["3_gl"] = np.array([0.5 - math.sqrt(3/5)/2, 0.5, 0.5 + math.sqrt(3/5)/2])

weights = {}
for _key, _x in _method_coefficients().items():
    _q = _NODES_OF[_key]
    weights[_key] = _x @ _rescale(_q) @ _moments(_q)

# number_of_exponentials -> (samples key, weights key), as selected by the
# reference's generate_simulator (superspinsim/generate_simulator.py:116-140)
METHODS = {1: ("1_gl", "2_1_gl"), 2: ("2_gl", "4_2_gl"), 3: ("2_gl", "4_3_gl"),
           5: ("3_gl", "6_5_gl"), 6: ("3_gl", "6_6_gl")}


def method(number_of_exponentials):
    """(weights K x Q, nodes Q) of the CF method with K exponentials."""
    if number_of_exponentials not in METHODS:
        raise ValueError("number_of_exponentials must be one of 1, 2, 3, 5, 6")
    s, w = METHODS[number_of_exponentials]
    return weights[w].copy(), samples[s].copy()
