"""The reference's own regression suite replayed through this package.

Every script of the reference's test/tests/ that checks its run against a
golden CSV (test/reference/*.csv), with that script's system, drive,
initial state and flags, run through this package's ``simspins`` at the
script's full length (10 us at 1 ns, F = 100).  The CSVs hold every 29th
value of the flattened (T, n, n, re/im) density; they are stored in full in
tests/golden/reference_csv.npz (make_golden.py csv).  Two checks:

* the reference's own pass criterion (test/tests/util.py, compare_density):
  sqrt(sum of squared differences) / number of values <= 1e-5;
* a max-abs bar per script (measured distances, with margin).  The
  seven scripts that wrote the CSVs, run with the reference's exponential
  (first-order Taylor, 2^-70 scaling, 70 squarings), reproduce them to
  about 1e-14, except qutrit-hyperfine (below).  The other scripts run
  different flags (rotating frame, other CF orders, residual arithmetic,
  kernel and unitary modes) against the same CSV; their distance is the
  difference between two integrators of the same equation.

The reference's kernel- and unitary-mode scripts read out of bounds in the
reference itself (generate_simulator.py:1026, :1047); here they run the
forms those modes intend and meet the same CSVs."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
import make_golden as mg  # noqa: E402  (system definitions; the reference is not imported)

pytestmark = pytest.mark.gpu

# script, csv, system, initial state, use_rotating, use_residual, K,
# use_kernel, use_unitary, use_hermitian (the -cpu twins of the reference's
# scripts run the same flags on its CPU path and are listed once)
SCRIPTS = [
    ("qubit-couple", "qubit-couple", "qubit", "q0", False, False, 1, False, False, True),
    ("qubit-couple-res", "qubit-couple", "qubit", "q0", False, True, 1, False, False, True),
    ("qubit-couple-res-ker", "qubit-couple", "qubit", "q0", False, True, 1, True, False, True),
    ("qubit-couple-res-ker-rot", "qubit-couple", "qubit", "q0", True, True, 1, True, False, True),
    ("qubit-couple-res-ker-rot-e5", "qubit-couple", "qubit", "q0", True, True, 5, True, False,
     True),
    ("qubit-couple-res-rot", "qubit-couple", "qubit", "q0", True, True, 1, False, False, True),
    ("qubit-couple-res-rot-e2", "qubit-couple", "qubit", "q0", True, True, 2, False, False, True),
    ("qubit-couple-res-rot-e5", "qubit-couple", "qubit", "q0", True, True, 5, False, False, True),
    ("qubit-couple-res-rot-e6", "qubit-couple", "qubit", "q0", True, True, 6, False, False, True),
    ("qubit-couple-res-rot-nh", "qubit-couple", "qubit", "q0", True, True, 1, False, False, False),
    ("qubit-hyperfine", "qubit-hyperfine", "qubit_hf", "e0", True, True, 1, False, False, True),
    ("qubit-t1-0K-res", "qubit-t1-0K", "t1_0K", "q1", False, True, 1, False, False, True),
    ("qubit-t1-0K-res-rot", "qubit-t1-0K", "t1_0K", "q1", True, True, 1, False, False, True),
    ("qubit-t1-mK-res", "qubit-t1-mK", "t1_mK", "q1", False, True, 1, False, False, True),
    ("qubit-t1-mK-res-rot", "qubit-t1-mK", "t1_mK", "q1", True, True, 1, False, False, True),
    ("qubit-t1-mK-res-rot-e2", "qubit-t1-mK", "t1_mK", "q1", True, True, 2, False, False, True),
    ("qubit-t1-mK-res-rot-e5", "qubit-t1-mK", "t1_mK", "q1", True, True, 5, False, False, True),
    ("qutrit-couple", "qutrit-couple", "qutrit", "t2", False, True, 1, False, False, True),
    ("qutrit-couple-ker", "qutrit-couple", "qutrit", "t2", False, True, 1, True, False, True),
    ("qutrit-couple-ker-rot", "qutrit-couple", "qutrit", "t2", True, True, 1, True, False, True),
    ("qutrit-couple-ker-rot-e5", "qutrit-couple", "qutrit", "t2", True, True, 5, True, False,
     True),
    ("qutrit-couple-rot", "qutrit-couple", "qutrit", "t2", True, True, 1, False, False, True),
    ("qutrit-couple-unitary", "qutrit-couple", "qutrit", "t2", True, True, 5, False, True, True),
    ("qutrit-couple-unital", "qutrit-couple-unital", "qutrit", "tu", False, True, 1, False, False,
     True),
    ("qutrit-couple-unital-ker", "qutrit-couple-unital", "qutrit", "tu", False, True, 1, True,
     False, True),
    ("qutrit-hyperfine", "qutrit-hyperfine", "qutrit_hf", "e0", True, True, 1, False, False,
     True),
]

# the scripts that wrote the CSVs
WRITERS = {"qubit-couple", "qubit-hyperfine", "qubit-t1-0K-res", "qubit-t1-mK-res",
           "qutrit-couple", "qutrit-couple-unital", "qutrit-hyperfine"}


def _system(name):
    t1 = mg.drive(28e6, 10e-3, t_end=mg.T1_END)
    return {"qubit": (mg.QUBIT, mg.drive(28e6, 10e-6)),
            "qubit_hf": (mg.QUBIT_HF, mg.drive(28e6, 10e-6)),
            "t1_0K": (mg.qubit_t1(0), t1),
            "t1_mK": (mg.qubit_t1(1e-3), t1),
            "qutrit": (mg.QUTRIT, mg.drive(7e6, 10e-6)),
            "qutrit_hf": (mg.QUTRIT_HF, mg.drive(7e6, 10e-6))}[name]


def _rho0(name):
    return {"q0": np.diag([1.0, 0.0]), "q1": np.diag([0.0, 1.0]),
            "t2": np.diag([0.0, 0.0, 1.0]), "tu": np.eye(3)/3,
            "e0": None}[name]


def _flat29(d):
    e = np.empty(d.shape + (2,))
    e[..., 0], e[..., 1] = d.real, d.imag
    return e.flatten()[::29]


def _run(script, expm):
    from superspinsim_gb300.sugar import simspins
    _, csv, system, rho, rot, res, K, ker, uni, herm = script
    spins, x = _system(system)
    rho0 = _rho0(rho)
    if rho0 is None:
        n = 4 if system == "qubit_hf" else 6
        rho0 = np.zeros((n, n))
        rho0[0, 0] = 1.0
    fns = [mg.channel_fn(x)] + [mg.channel_fn(mg.ZERO)]*3
    _, d = simspins(fns, 0, 10e-6, 1e-9, spins, [{}], {}, rho0.astype(np.float64),
                    number_of_exponentials=K, number_of_fine_divisions=100,
                    use_rotating=rot, use_residual=res, use_kernel=ker, use_unitary=uni,
                    use_hermitian=herm, expm=expm)
    return d


# Max-abs distance from the CSV, per script.  qubit-couple.csv was written
# in plain (non-residual) lab-frame arithmetic at CF2:1, whose squarings
# lose the small terms; every other flag set, and the same flags with the
# accurate exponential, lands 2.4-2.6e-6 from it after 10 us.  The T1 runs drive a 10 mT pi
# pulse (280 MHz Rabi) that ends at 1.79 ns, inside a 10 ps fine step:
# CF orders 1, 2 and 5 integrate that jump differently (the K = 2 run
# equals the reference's own K = 2 output, fixture qubit_t1_mK_rot_e2).
# qutrit-hyperfine.csv (the 36 x 36 lab-frame run its script falls back
# to: its rotating frame is singular) lies 3.9e-7 from this package's runs
# with either exponential, which agree with each other to 1e-12.
BARS = {
    "qubit-couple": 5e-6, "qubit-couple-res": 5e-6, "qubit-couple-res-ker": 5e-6,
    "qubit-couple-res-ker-rot": 5e-6, "qubit-couple-res-ker-rot-e5": 5e-6,
    "qubit-couple-res-rot": 5e-6, "qubit-couple-res-rot-e2": 5e-6,
    "qubit-couple-res-rot-e5": 5e-6, "qubit-couple-res-rot-e6": 5e-6,
    "qubit-couple-res-rot-nh": 5e-6,
    "qubit-hyperfine": 1e-12,
    "qubit-t1-0K-res": 1e-12, "qubit-t1-0K-res-rot": 5e-6,
    "qubit-t1-mK-res": 1e-12, "qubit-t1-mK-res-rot": 5e-6,
    "qubit-t1-mK-res-rot-e2": 5e-3, "qubit-t1-mK-res-rot-e5": 5e-3,
    "qutrit-couple": 1e-12, "qutrit-couple-ker": 1e-12, "qutrit-couple-ker-rot": 5e-8,
    "qutrit-couple-ker-rot-e5": 5e-8, "qutrit-couple-rot": 5e-8, "qutrit-couple-unitary": 5e-8,
    "qutrit-couple-unital": 1e-12, "qutrit-couple-unital-ker": 1e-12,
    "qutrit-hyperfine": 1e-6,
}

_RUNS = {}


def _cached(script, expm):
    key = (script[0], expm)
    if key not in _RUNS:
        _RUNS[key] = _flat29(_run(script, expm))
    return _RUNS[key]


@pytest.fixture(scope="module")
def csvs():
    with np.load(os.path.join(GOLDEN, "reference_csv.npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("script", SCRIPTS, ids=[s[0] for s in SCRIPTS])
def test_reference_script(script, csvs):
    ref = csvs[script[1]]
    this = _cached(script, "taylor")
    assert this.shape == ref.shape
    diff = this - ref
    assert np.all(np.isfinite(this))
    assert np.sqrt(np.sum(diff**2))/this.size <= 1e-5      # the reference's criterion
    assert np.abs(diff).max() <= BARS[script[0]], np.abs(diff).max()


@pytest.mark.parametrize("script", [s for s in SCRIPTS if s[0] in WRITERS],
                         ids=[s[0] for s in SCRIPTS if s[0] in WRITERS])
def test_csv_writers_reproduce_their_csv(script, csvs):
    """The scripts that wrote the CSVs, with the reference's own
    exponential: the CSV to 1e-13 over the whole run (qutrit-hyperfine:
    see BARS).  In residual arithmetic the package's default exponential
    lands within 1e-11 of it; qubit-couple's plain arithmetic (the identity
    added before the 70 squarings) loses the small terms, which is why every
    other flag set lies 2.4e-6 from qubit-couple.csv."""
    ref = csvs[script[1]]
    this = _cached(script, "reference")
    bar = BARS[script[0]] if script[0] == "qutrit-hyperfine" else 1e-13
    assert np.abs(this - ref).max() <= bar
    if script[5]:
        assert np.abs(this - _cached(script, "taylor")).max() <= 1e-11
