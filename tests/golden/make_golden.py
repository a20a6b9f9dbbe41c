"""Generate the golden fixtures under ``tests/golden/`` from the reference.

This script is test infrastructure.  It imports the unmodified reference
package (monashNV/superspinsim 1.3.2) from the checkout named by the
environment variable ``SSS_REFERENCE`` (required) and runs its own CPU
path.  numba and qutip are not
installed here, so a small import shim stands in for them:

* ``numba.jit`` becomes the identity and ``numba.prange`` becomes ``range``
  (the reference's CPU kernels then run as plain Python loops, with Python's
  float64 arithmetic and no fast-math reassociation);
* ``numba.cuda`` is a sequential stand-in that runs each of the
  reference's GPU kernels once per thread index in Python (``nc.fma`` is
  an unfused multiply-add).  Runs use the reference's GPU branch by
  default -- the branch that produced its golden CSVs -- because its CPU
  rotating-frame branch indexes out of bounds
  (``superspinsim/generate_simulator.py:985``, loop bound ``doubles_size``
  instead of ``singles_size``); cases marked ``path="cpu"`` take the CPU
  branch (``use_cuda=False``) to pin it too;
* ``qutip.Qobj`` is an empty class (only used in ``isinstance`` checks,
  ``superspinsim/sugar.py:181``).

For each case the fixture stores the reference's generators
(``generate_atoms``, ``superspinsim/generate_generators.py:19-166``), its
vectorisation map, the generalised-rotating-frame arrays when used
(``make_rotating``, ``:2491-2519``), the coefficient program in this
project's segment format, and the density operators returned by
``simulate`` (``superspinsim/generate_simulator.py:1508-2200``) on a short
window.  Where the case is one of the reference's golden regression tests,
the leading values of its CSV (``test/reference/*.csv``) are stored too.

Run:  SSS_REFERENCE=<reference checkout> python tests/golden/make_golden.py
                                                    (about 5 minutes, 1 core)
      python tests/golden/make_golden.py modes      (unitary / kernel mode arrays)
      python tests/golden/make_golden.py csv        (the golden CSVs in full)
      python tests/golden/make_golden.py fullrun    (full-length runs of the
          reference's algorithm through the oracle's reference mode: NV-7
          over 400,000 steps, NV-21 over 104; about 30 minutes on 8 cores;
          no reference checkout needed)
"""
import math
import os
import sys
import time as _time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("SSS_REFERENCE")

_SHIM = {
    "numba/__init__.py": (
        "def jit(*args, **kwargs):\n"
        "    if len(args) == 1 and callable(args[0]):\n"
        "        return args[0]\n"
        "    return lambda f: f\n"
        "prange = range\n"
        "from . import core\n"),
    "numba/core/__init__.py": "from . import errors\n",
    "numba/core/errors.py":
        "class NumbaPerformanceWarning(Warning):\n    pass\n",
    "qutip/__init__.py": "class Qobj:\n    pass\n",
    # Sequential stand-in for numba.cuda: each kernel launch runs its
    # Python body once per (block, thread) index, in order.  The
    # reference's kernels use no shared memory or barriers (the only uses
    # are in commented-out code), and none of them writes an array that
    # another thread of the same launch reads, so sequential execution
    # gives the same result as a GPU.  nc.fma is an unfused a*b + c.
    "numba/cuda/__init__.py": (
        "import numpy as _np\n"
        "class _Dim:\n"
        "    def __init__(self):\n"
        "        self.x = self.y = self.z = 0\n"
        "threadIdx, blockIdx, blockDim = _Dim(), _Dim(), _Dim()\n"
        "def fma(a, b, c):\n"
        "    return a*b + c\n"
        "class DeviceArray(_np.ndarray):\n"
        "    def copy_to_host(self):\n"
        "        return _np.array(self)\n"
        "def device_array(shape, dtype=_np.float64):\n"
        "    return _np.zeros(shape, dtype).view(DeviceArray)\n"
        "def to_device(a):\n"
        "    return _np.array(a).view(DeviceArray)\n"
        "def _dims(d):\n"
        "    d = tuple(d) if isinstance(d, (tuple, list)) else (d,)\n"
        "    return tuple(int(v) for v in d) + (1,)*(3 - len(d))\n"
        "class _Kernel:\n"
        "    def __init__(self, f):\n"
        "        self.f = f\n"
        "    def __getitem__(self, cfg):\n"
        "        grid, block = _dims(cfg[0]), _dims(cfg[1])\n"
        "        def launch(*args):\n"
        "            blockDim.x, blockDim.y, blockDim.z = block\n"
        "            for bz in range(grid[2]):\n"
        "                for by in range(grid[1]):\n"
        "                    for bx in range(grid[0]):\n"
        "                        blockIdx.x, blockIdx.y, blockIdx.z = bx, by, bz\n"
        "                        for tz in range(block[2]):\n"
        "                            for ty in range(block[1]):\n"
        "                                for tx in range(block[0]):\n"
        "                                    threadIdx.x = tx\n"
        "                                    threadIdx.y = ty\n"
        "                                    threadIdx.z = tz\n"
        "                                    self.f(*args)\n"
        "        return launch\n"
        "def jit(f=None, device=False, **kwargs):\n"
        "    if f is None:\n"
        "        return lambda g: jit(g, device=device)\n"
        "    return f if device else _Kernel(f)\n"),
}


def install_shim():
    # the shim (and the HOME the reference's mesolve writes its temporary
    # module under) live in tests/golden/.shim, which git ignores
    root = os.path.join(HERE, ".shim")
    os.makedirs(root, exist_ok=True)
    os.environ["HOME"] = os.path.join(root, "home")
    for rel, text in _SHIM.items():
        path = os.path.join(root, rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            f.write(text)
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "superspinsim")):
        raise SystemExit("set SSS_REFERENCE to a checkout of monashNV/superspinsim 1.3.2 "
                         "(the directory that holds superspinsim/)")
    sys.path.insert(0, REFERENCE)
    sys.path.insert(0, root)


# Coefficient programs ------------------------------------------------------
# A program is, per control channel (x, y, z field in tesla; r = optical
# excitation), a list of segments (t_end, offset, amplitude, frequency,
# phase): for t < t_end (first match) the channel is
# offset + amplitude*cos(tau*frequency*t + phase); after the last segment
# it is 0.


def channel_fn(segs):
    segs = [tuple(float(v) for v in s) for s in segs]

    def fn(t):
        for t_end, off, amp, freq, ph in segs:
            if t < t_end:
                return off + amp*math.cos(math.tau*freq*t + ph)
        return 0.0
    return fn


def drive(freq, amp, t_end=1.0, phase=0.0, offset=0.0):
    return [(t_end, offset, amp, freq, phase)]


def const(value, t_end=1.0):
    return [(t_end, value, 0.0, 0.0, 0.0)]


def program_array(channels):
    """Pack the 4 channels as a (4, S, 5) float64 array (S = max segments,
    missing segments padded with t_end = -inf so they never match)."""
    smax = max(1, max(len(c) for c in channels))
    out = np.zeros((4, smax, 5))
    out[:, :, 0] = -np.inf
    for g, segs in enumerate(channels):
        for s, seg in enumerate(segs):
            out[g, s, :] = seg
    return out


# Cases --------------------------------------------------------------------
B0 = np.array([0, 0, 1e-3])
QUBIT = [[{"S": 1/2, "g": 2.0, "B0": B0}]]
QUTRIT = [[{"S": 1, "g": -1/2, "D": 72, "B0": B0}]]


def qubit_t1(temp):
    return [[{"S": 1/2, "g": 2.0, "B0": B0, "TS1": 1e-6, "T": temp}]]


QUBIT_HF = [[{"S": 1/2, "g": 2.0, "B0": B0, "I": 1/2, "g": 1.0, "A": 2e9}]]
QUTRIT_HF = [[{"S": 1, "g": -1/2, "D": 72, "B0": B0, "I": 1/2, "gI": 1.0,
               "A": 2e9}]]


def spin1_c1():
    """Spin-1 NV ground state, 10 mT along z, Lindblad dephasing and T1."""
    return [[{"S": 1, "g": 28.025e9/13996244917.1, "D": math.tau*2.870e9,
              "B0": np.array([0, 0, 0.01]), "TS2": 1e-6, "TS1": 1e-3,
              "T": 293.15}]]


T1_END = 1/(2*10e-3*28e9)
ZERO = const(0.0)


def coherent_chain():
    """A qubit, a qutrit and a qubit in three blocks joined by coherent
    couplings: the first qubit's m = +1/2 to the qutrit's m = 0 at a
    constant 30 MHz (Vc), the qutrit's m = 0 on to the second qubit's
    m = -1/2 at 20 MHz times the fourth channel (Vr).  The qubits are joined only
    through the qutrit, so their mutual coherences are allowed by the
    transitive closure.  (The spins differ along the chain: the reference
    numbers the couplings wrongly after a coupling between equal spins
    that has no "rel" rate, and raises at the next one.)"""
    spins = [[{"S": 1/2, "g": 2.0, "B0": B0}],
             [{"S": 1, "g": -1/2, "D": 72, "B0": B0}],
             [{"S": 1/2, "g": 2.0, "B0": B0}]]
    groups = {
        ((0, 0), (1, 0)): {"coh": [{"ini": 1/2, "fin": 0, "amp": math.tau*30e6}]},
        ((1, 0), (2, 0)): {"coh": [{"ini": 0, "fin": -1/2, "amp": math.tau*20e6,
                                    "con": True}]},
    }
    return spins, [{}, {}, {}], groups


def hbn_bell():
    """A pair of spin-1/2 atoms in one block (a hBN-like triplet pair) and a
    singlet block: the singlet decays into the Bell states of the pair
    (psi at 20 /us, phi at 10 /us) and the pair decays back (psi at 3 /us,
    phi at 1 /us)."""
    pair = [{"S": 1/2, "g": 2.0, "B0": B0, "TS2": 1e-6},
            {"S": 1/2, "g": 2.0, "B0": B0}]
    spins = [pair, [{"S": 0}]]
    groups = {
        ((1, 0), (0, 0)): {"psi_gets_e": 2e7, "phi_gets_e": 1e7},
        ((0, 0), (1, 0)): {"g_gets_psi": 3e6, "g_gets_phi": 1e6},
    }
    return spins, [{}, {}], groups


def cases():
    q_drive = drive(28e6, 10e-6)
    t_drive = drive(7e6, 10e-6)
    c1_drive = drive(2.870e9 + 28.025e9*0.01 + 5e6, 10e6/28.025e9)
    rho_q0 = np.diag([1.0, 0.0]).astype(complex)
    rho_q1 = np.diag([0.0, 1.0]).astype(complex)
    rho_t2 = np.diag([0.0, 0.0, 1.0]).astype(complex)
    rho_tu = np.eye(3, dtype=complex)/3
    rho_hf = np.zeros((4, 4), complex)
    rho_hf[0, 0] = 1
    rho_c1 = np.diag([0.0, 1.0, 0.0]).astype(complex)
    base = dict(spin_interactions=[{}], group_interactions={},
                use_kernel=False, use_unitary=False, use_incoherent=True,
                R=35)
    out = [
        dict(name="qubit_couple", csv="qubit-couple", spins=QUBIT,
             ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_q0, t=(0, 20e-9, 1e-9),
             rot=False, res=False, K=1, F=100),
        dict(name="qubit_couple_res_e2", csv="qubit-couple", spins=QUBIT,
             ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_q0, t=(0, 20e-9, 1e-9),
             rot=False, res=True, K=2, F=10),
        dict(name="qubit_couple_res_e2_cpu", csv="qubit-couple",
             spins=QUBIT, ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_q0,
             t=(0, 20e-9, 1e-9), rot=False, res=True, K=2, F=10,
             path="cpu"),
        dict(name="qubit_couple_res_e5", csv="qubit-couple", spins=QUBIT,
             ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_q0, t=(0, 10e-9, 1e-9),
             rot=False, res=True, K=5, F=10),
        dict(name="qubit_couple_res_e3_e6", csv="qubit-couple", spins=QUBIT,
             ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_q0, t=(0, 6e-9, 1e-9),
             rot=False, res=True, K=3, F=10, K2=6),
        dict(name="qubit_t1_0K", csv="qubit-t1-0K", spins=qubit_t1(0),
             ch=[drive(28e6, 10e-3, t_end=T1_END), ZERO, ZERO, ZERO],
             rho0=rho_q1, t=(0, 20e-9, 1e-9), rot=False, res=True, K=1,
             F=100),
        dict(name="qubit_t1_mK", csv="qubit-t1-mK", spins=qubit_t1(1e-3),
             ch=[drive(28e6, 10e-3, t_end=T1_END), ZERO, ZERO, ZERO],
             rho0=rho_q1, t=(0, 20e-9, 1e-9), rot=False, res=True, K=1,
             F=100),
        dict(name="qutrit_couple", csv="qutrit-couple", spins=QUTRIT,
             ch=[t_drive, ZERO, ZERO, ZERO], rho0=rho_t2, t=(0, 5e-9, 1e-9),
             rot=False, res=True, K=1, F=100),
        dict(name="qutrit_couple_unital", csv="qutrit-couple-unital",
             spins=QUTRIT, ch=[t_drive, ZERO, ZERO, ZERO], rho0=rho_tu,
             t=(0, 5e-9, 1e-9), rot=False, res=True, K=1, F=100),
        dict(name="qubit_hyperfine", csv="qubit-hyperfine", spins=QUBIT_HF,
             ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_hf, t=(0, 1e-9, 1e-9),
             rot=True, res=True, K=1, F=100),
        dict(name="qubit_couple_rot_e5", csv="qubit-couple", spins=QUBIT,
             ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_q0, t=(0, 10e-9, 1e-9),
             rot=True, res=True, K=5, F=10),
        dict(name="qubit_couple_rot_e1_nores", csv="qubit-couple",
             spins=QUBIT, ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_q0,
             t=(0, 10e-9, 1e-9), rot=True, res=False, K=1, F=10),
        # the reference's qubit-t1-0K-res-rot.py and qubit-t1-mK-res-rot-e2.py:
        # the rotating frame with decay (damped e^{L0 h} blocks)
        dict(name="qubit_t1_0K_rot", csv=None, spins=qubit_t1(0),
             ch=[drive(28e6, 10e-3, t_end=T1_END), ZERO, ZERO, ZERO],
             rho0=rho_q1, t=(0, 20e-9, 1e-9), rot=True, res=True, K=1, F=100),
        dict(name="qubit_t1_mK_rot_e2", csv=None, spins=qubit_t1(1e-3),
             ch=[drive(28e6, 10e-3, t_end=T1_END), ZERO, ZERO, ZERO],
             rho0=rho_q1, t=(0, 20e-9, 1e-9), rot=True, res=True, K=2, F=100),
        # the reference's test qubit-couple-res-rot-nh.py: the complex
        # (non-Hermitian) basis, N = 2 n^2, no vectorisation map
        dict(name="qubit_couple_rot_nh", csv="qubit-couple", spins=QUBIT,
             ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_q0, t=(0, 10e-9, 1e-9),
             rot=True, res=True, K=1, F=100, herm=False),
        dict(name="qubit_couple_nh", csv="qubit-couple", spins=QUBIT,
             ch=[q_drive, ZERO, ZERO, ZERO], rho0=rho_q0, t=(0, 10e-9, 1e-9),
             rot=False, res=True, K=2, F=10, herm=False),
        dict(name="spin1_c1", csv=None, spins=spin1_c1(),
             ch=[c1_drive, ZERO, ZERO, ZERO], rho0=rho_c1,
             t=(0, 1e-9, 1e-9), rot=False, res=True, K=2, F=100,
             use_incoherent=False),
        dict(name="coherent_chain", csv=None, spins=coherent_chain()[0],
             spin_interactions=coherent_chain()[1],
             group_interactions=coherent_chain()[2],
             ch=[q_drive, ZERO, ZERO, const(0.5)],
             rho0=np.diag([1.0, 0, 0, 0, 0, 0, 0]).astype(complex),
             t=(0, 4e-9, 1e-9), rot=False, res=True, K=2, F=10, path="cpu"),
        dict(name="hbn_bell", csv=None, spins=hbn_bell()[0],
             spin_interactions=hbn_bell()[1], group_interactions=hbn_bell()[2],
             ch=[q_drive, ZERO, ZERO, ZERO],
             rho0=np.diag([0.0, 0, 0, 0, 1.0]).astype(complex),
             t=(0, 10e-9, 1e-9), rot=False, res=True, K=2, F=20, path="cpu"),
        dict(name="qutrit_hyperfine", csv="qutrit-hyperfine",
             spins=QUTRIT_HF, ch=[t_drive, ZERO, ZERO, ZERO],
             rho0=np.diag([1.0, 0, 0, 0, 0, 0]).astype(complex),
             t=None, rot=True, res=True, K=1, F=100),
    ]
    for c in out:
        for k, v in base.items():
            c.setdefault(k, v)
    return out


def nv7_case(name, use_incoherent, t, F, K=2, extra=None):
    """The 7-level NV model (reference ``models.nv_7``) at B = 5 mT along z
    with the rates of the 7-level ODMR workload, driven by an x field
    at the ms=0 -> +1 resonance plus 5 MHz detuning, laser at 10/65.9 of
    saturation (pump rate 10 /us)."""
    from superspinsim import models, params
    P = nv7_params(params)
    spins, inter, groups = models.nv_7(np.array([0, 0, 5e-3]), params=P)
    f_res = 2.870e9 + 28.025e9*5e-3
    amp = 5e6/28.025e9
    rho0 = np.zeros((7, 7), complex)
    rho0[1, 1] = 1.0
    c = dict(name=name, csv=None, spins=spins, spin_interactions=inter,
             group_interactions=groups,
             ch=[drive(f_res + 5e6, amp), ZERO, ZERO, const(10/65.9)],
             rho0=rho0, t=t, rot=False, res=True, K=K, F=F,
             use_incoherent=use_incoherent, use_kernel=False,
             use_unitary=False, R=35)
    if extra:
        c.update(extra)
    return c


def nv7_params(params):
    """The reference's parameter module with the 7-level ODMR workload's
    rates: ground D = 2.870 GHz, excited D = 1.42 GHz, spin-conserving
    optical decay 65.9 /us, ISC 11 /us (ms=0) and 80 /us (ms=+-1) into the
    singlet, singlet decay 3.0 /us to ms=0 and 2.6 /us to ms=+-1."""
    import copy
    import types
    P = types.SimpleNamespace()
    P.fundamental = params.fundamental
    P.standards = params.standards

    class ground(params.nv.room.ground):
        zfs_longitudinal = 2.870e9

    class excited(params.nv.room.excited):
        zfs_longitudinal = 1.42e9

    class optical(params.nv.room.optical):
        conserving = 65.9e6
        nonconserving = None

    class isc(params.nv.room.isc):
        s_gets_z = 11e6
        s_gets_pm = 80e6
        z_gets_s = 3.0e6
        pm_gets_s = 2.6e6

    class room:
        pass
    room.ground, room.excited, room.optical, room.isc = \
        ground, excited, optical, isc

    class nv:
        pass
    nv.room = room
    P.nv = nv
    return copy.copy(P)


def nv21_case():
    """The 21-level NV (14N spin 1 in every orbital manifold, as in the
    reference's legacy generate_21, generate_generators.py:2944-3028) at
    50 mT with the 7-level ODMR rates and the ground-state 14N constants
    A_par = -2.16 MHz, A_perp = -2.70 MHz, P = -4.95 MHz.  Generators only:
    the reference's simulate is pure Python under the shim and too slow at
    N = 441."""
    from superspinsim import params
    P = nv7_params(params)
    g, e = P.nv.room.ground, P.nv.room.excited
    B0 = np.array([0, 0, 0.05])
    T = params.standards.lab.ntp.temperature
    ground = {"S": 1, "g": g.g_longitudinal, "g_perp": g.g_transverse,
              "D": math.tau*g.zfs_longitudinal, "TS1": g.thermalisation_time,
              "TS2": g.dephasing_time, "I": 1, "gN": g.g_N_14N_longitudinal,
              "P": math.tau*(-4.95e6), "TI1": g.thermalisation_time_14N,
              "TI2": g.dephasing_time_14N, "A": math.tau*(-2.16e6),
              "A_perp": math.tau*(-2.70e6), "B0": B0, "T": T}
    excited = {"S": 1, "g": e.g_longitudinal, "D": math.tau*e.zfs_longitudinal,
               "TS1": e.thermalisation_time, "TS2": e.dephasing_time, "I": 1,
               "gN": e.g_N_14N_longitudinal,
               "P": math.tau*e.nuclear_quadrupole_14N_longitudinal,
               "TI1": e.thermalisation_time_14N, "TI2": e.dephasing_time_14N,
               "A": math.tau*e.hyperfine_14N_longitudinal,
               "A_perp": math.tau*e.hyperfine_14N_transverse, "B0": B0, "T": T}
    singlet = {"S": 0, "I": 1, "gN": g.g_N_14N_longitudinal,
               "P": math.tau*(-4.95e6), "TI1": g.thermalisation_time_14N,
               "TI2": g.dephasing_time_14N, "B0": B0, "T": T}
    from superspinsim import models
    _, _, groups = models.nv_7(B0, params=P)
    return [[ground], [excited], [singlet]], [{}, {}, {}], groups


def save_nv21():
    from superspinsim.generate_generators import generate_atoms
    spins, inter, groups = nv21_case()
    t = _time.time()
    g, vm = generate_atoms(spins, inter, groups, False, True, False)
    gens = np.array([g["generators"][k] for k in ["L0", "Gx", "Gy", "Gz", "Gr"]])
    np.savez_compressed(os.path.join(HERE, "nv21_n441.npz"), generators=gens,
                        vectorisation_map=vm)
    print(f"nv21_n441: N={gens.shape[1]} {_time.time() - t:.1f} s", flush=True)


def mesolve_case():
    """A driven, damped qubit through the reference's QuTiP-style front end
    (superspinsim/sugar.py:21-161), rotating frame (its default).  The jump
    operators are static: the reference's time-dependent jump path wraps
    its coefficient in a closure over a name it then rebinds to the closure
    itself (sugar.py:124-135) and recurses without end."""
    sz = np.diag([1.0, -1.0]).astype(complex)
    sx = np.array([[0, 1], [1, 0]], complex)
    sm = np.array([[0, 0], [1, 0]], complex)
    H = [math.tau*30e6*sz/2,
         [sx, lambda t: math.tau*4e6*math.cos(math.tau*30e6*t)]]
    c_ops = [math.sqrt(2e6)*sm, math.sqrt(1e5)*sz]
    rho0 = np.array([[1, 0], [0, 0]], complex)
    return H, c_ops, rho0


def save_mesolve():
    from superspinsim import mesolve
    H, c_ops, rho0 = mesolve_case()
    t = _time.time()
    _, d = mesolve(H, rho0, 0.0, 20e-9, 1e-9, c_ops=c_ops, number_of_exponentials=5,
                   number_of_fine_divisions=10)
    np.savez_compressed(os.path.join(HERE, "mesolve_qubit.npz"), density=d)
    print(f"mesolve_qubit: {_time.time() - t:.1f} s", flush=True)


def build_generators(c):
    from superspinsim.generate_generators import generate_atoms, \
        make_rotating
    g, vmap = generate_atoms(
        c["spins"], c["spin_interactions"], c["group_interactions"],
        False, c.get("herm", True), c["use_incoherent"])
    gens = [g["generators"][k] for k in ["L0", "Gx", "Gy", "Gz", "Gr"]]
    out = dict(generators=np.array(gens), vectorisation_map=vmap)
    if c["rot"]:
        gr, V, Vi, D, S = make_rotating(gens[0], gens[1:])
        out.update(generators_rotating=np.array(gr), vectors_real=V,
                   inv_vectors_real=Vi, doubles=D.reshape(-1, 2),
                   singles=S)
    return out


def run_reference(c, K=None):
    from superspinsim import simspins
    fns = [channel_fn(s) for s in c["ch"]]
    t0, tf, dt = c["t"]
    _, dens = simspins(
        fns, t0, tf, dt, c["spins"], c["spin_interactions"],
        c["group_interactions"], c["rho0"],
        number_of_exponentials=K or c["K"],
        number_of_fine_divisions=c["F"],
        number_of_quadratic_repeats=c["R"], use_rotating=c["rot"],
        use_residual=c["res"], use_kernel=False, use_unitary=False,
        use_cuda=(c.get("path", "gpu") == "gpu"),
        use_hermitian=c.get("herm", True), use_incoherent=c["use_incoherent"])
    return dens


def csv_prefix(name, count=400):
    path = os.path.join(REFERENCE, "test", "reference", name + ".csv")
    return np.loadtxt(path, delimiter=",")[:count]


def save_case(c, extra_runs=()):
    t_start = _time.time()
    arrays = build_generators(c)
    arrays["program"] = program_array(c["ch"])
    arrays["rho0"] = c["rho0"]
    meta = dict(rot=c["rot"], res=c["res"], K=c["K"], F=c["F"], R=c["R"],
                use_incoherent=c["use_incoherent"],
                path=c.get("path", "gpu"), herm=c.get("herm", True))
    if c["t"] is not None:
        arrays["times"] = np.array(c["t"], dtype=float)
        arrays["density"] = run_reference(c)
        for K2 in extra_runs:
            arrays[f"density_K{K2}"] = run_reference(c, K=K2)
    if c["csv"]:
        arrays["csv_prefix"] = csv_prefix(c["csv"])
    for k, v in meta.items():
        arrays["meta_" + k] = np.array(v)
    path = os.path.join(HERE, c["name"] + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"{c['name']}: N={arrays['generators'].shape[1]} "
          f"{_time.time() - t_start:.1f} s", flush=True)


def save_reference_csvs():
    """The reference's golden regression vectors in full
    (``test/reference/*.csv``: every 29th value of the flattened
    (T, n, n, re/im) density of a 10 us run at 1 ns, F = 100), as
    ``reference_csv.npz``, keyed by CSV name."""
    names = ["qubit-couple", "qubit-hyperfine", "qubit-t1-0K", "qubit-t1-mK",
             "qutrit-couple", "qutrit-couple-unital", "qutrit-hyperfine"]
    arrays = {}
    for name in names:
        path = os.path.join(REFERENCE, "test", "reference", name + ".csv")
        arrays[name] = np.loadtxt(path, delimiter=",")
    np.savez_compressed(os.path.join(HERE, "reference_csv.npz"), **arrays)
    print("reference_csv:", {k: v.shape[0] for k, v in arrays.items()}, flush=True)


def save_modes():
    """Operator (unitary) generators, elimination/duplication matrices and
    the equivalence-class projection of the reference for the qubit, qutrit
    and hyperfine systems (``generate_generators.py:120-139``, ``find_kernel``
    :2691-2719), as ``modes_<system>.npz``."""
    from superspinsim.generate_generators import generate_atoms, find_kernel
    for name, spins in (("qubit", QUBIT), ("qutrit", QUTRIT), ("qubit_hf", QUBIT_HF)):
        arrays = {}
        g, vmap = generate_atoms(spins, [{}], {}, True, True, True)
        for k in ("H0", "Gx", "Gy", "Gz", "Gr"):
            arrays["unitary_" + k] = g["unitary"][k]
        arrays["elimination"] = g["elimination"]["elimination"]
        arrays["duplication"] = g["elimination"]["duplication"]
        arrays["vectorisation_map"] = vmap
        g, vmap = generate_atoms(spins, [{}], {}, False, True, True)
        gens = [g["generators"][k] for k in ["L0", "Gx", "Gy", "Gz", "Gr"]]
        full, image, gens_image = find_kernel(gens)
        arrays["generators"] = np.array(gens)
        arrays["full_projection"] = full
        arrays["image_projection"] = image
        arrays["generators_image"] = np.array(gens_image)
        np.savez_compressed(os.path.join(HERE, f"modes_{name}.npz"), **arrays)
        print(f"modes_{name}: N={gens[0].shape[0]} r={image.shape[1]}", flush=True)


def save_quadratures():
    """The reference's Gauss-Legendre nodes and commutator-free weights
    (``superspinsim/quadratures.py:10-50``)."""
    from superspinsim.quadratures import samples, weights
    arrays = {}
    for k, v in samples.items():
        arrays["samples_" + k] = np.asarray(v, dtype=np.float64)
    for k, v in weights.items():
        arrays["weights_" + k] = np.asarray(v, dtype=np.float64)
    np.savez(os.path.join(HERE, "quadratures.npz"), **arrays)


# Full-length runs of the reference's algorithm -----------------------------
# The oracle's reference mode reproduces the reference's simulate bit for
# bit on every fixture above (tests/test_oracle_golden.py), so it stands in
# for the reference on runs far too long for the shimmed Python: the whole
# 400,000-step NV-7 ODMR trajectory and a 104-step window of the NV-21
# (441 x 441) sweep.  Both use the reference's own generators (the nv7_n49
# and nv21_n441 fixtures) and its quadrature tables (quadratures.npz); they
# need no reference checkout.

F_RES_NV7 = 2.870e9 + 28.025e9*5e-3
F_RES_NV21 = 2.870e9 + 28.025e9*0.05


def odmr_program(freq, rabi=5e6, laser=10/65.9):
    """x drive of Rabi frequency `rabi` at `freq`, laser pumping at `laser`
    of saturation, for all time (the ODMR workloads' programs)."""
    p = np.zeros((4, 1, 5))
    p[:, :, 0] = np.inf
    p[0, 0, 2:4] = [rabi/28.025e9, freq]
    p[3, 0, 1] = laser
    return p


def _flat(rho, vm):
    out = np.zeros(vm.shape[0])
    for i, (y, x, c) in enumerate(vm):
        out[i] = rho[y, x].imag if c else rho[y, x].real
    return out


def save_fullruns(which=("nv7_fullrun", "nv21_window")):
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import oracle
    with np.load(os.path.join(HERE, "quadratures.npz")) as z:
        W, nodes = z["weights_4_2_gl"], z["samples_2_gl"]
    if "nv7_fullrun" in which:
        # the 1024-frequency sweep's trajectory 512 (the one nearest the
        # ms=0 -> +1 line), 2 us at 5 ps: T = 2000 samples of 1 ns, F = 200
        with np.load(os.path.join(HERE, "nv7_n49.npz")) as z:
            gens, vm = z["generators"], z["vectorisation_map"]
        freqs = F_RES_NV7 + np.linspace(-30e6, 30e6, 1024)
        index = 512
        prog = odmr_program(freqs[index])
        rho = np.zeros((7, 7), complex)
        rho[1, 1] = 1.0
        T, dt, F = 2000, 1e-9, 200
        t = _time.time()
        _, out = oracle.simulate(gens, rho, 0.0, T*dt + 1e-13, dt, prog, K=2, W=W, nodes=nodes,
                                 F=F, vectorisation_map=vm, mode="reference", flat_out=True)
        w = np.zeros(vm.shape[0])
        for i, (y, x, c) in enumerate(vm):
            if y == x and c == 0 and y in (3, 4, 5):
                w[i] = 65.9e6
        keep = np.arange(99, T, 100)
        np.savez_compressed(os.path.join(HERE, "nv7_fullrun.npz"), index=index,
                            freqs=freqs, program=prog, rho0=_flat(rho, vm), T=T, dt=dt, F=F,
                            fluorescence=out @ w, readout_weights=w, kept_samples=keep,
                            states=out[keep])
        print(f"nv7_fullrun: {T*F} steps in {_time.time() - t:.0f} s", flush=True)
    if "nv21_window" in which:
        # four trajectories of the 256-frequency NV-21 sweep, 8 samples of
        # 65 ps with F = 13 (104 steps of 5 ps), every sample's state kept
        with np.load(os.path.join(HERE, "nv21_n441.npz")) as z:
            gens, vm = z["generators"], z["vectorisation_map"]
        freqs = F_RES_NV21 + np.linspace(-30e6, 30e6, 256)
        index = np.array([0, 100, 128, 255])
        progs = np.stack([odmr_program(freqs[i]) for i in index])
        rho = np.zeros((21, 21), complex)
        for k in range(3, 6):
            rho[k, k] = 1/3
        T, dt, F = 8, 65e-12, 13
        t = _time.time()
        _, out = oracle.simulate(gens, np.stack([rho]*len(index)), 0.0, T*dt + 1e-15, dt, progs,
                                 K=2, W=W, nodes=nodes, F=F, vectorisation_map=vm,
                                 mode="reference", flat_out=True)
        np.savez_compressed(os.path.join(HERE, "nv21_window.npz"), index=index, freqs=freqs,
                            programs=progs, rho0=_flat(rho, vm), T=T, dt=dt, F=F, states=out)
        print(f"nv21_window: {len(index)} x {T*F} steps in {_time.time() - t:.0f} s", flush=True)


def main():
    only = set(sys.argv[1:])
    if only & {"nv7_fullrun", "nv21_window", "fullrun"}:
        save_fullruns(tuple(only) if "fullrun" not in only else ("nv7_fullrun", "nv21_window"))
        return
    install_shim()
    if "modes" in only:
        save_modes()
        return
    if "csv" in only:
        save_reference_csvs()
        return
    save_quadratures()
    for c in cases():
        if only and c["name"] not in only:
            continue
        save_case(c, extra_runs=(c["K2"],) if "K2" in c else ())
    extra = [
        nv7_case("nv7_n49", False, (0, 10e-12, 10e-12), F=2),
        nv7_case("nv7_n19", True, (0, 20e-12, 10e-12), F=2),
    ]
    for c in extra:
        if only and c["name"] not in only:
            continue
        save_case(c)
    if not only or "nv21_n441" in only:
        save_nv21()
    if not only or "mesolve_qubit" in only:
        save_mesolve()


if __name__ == "__main__":
    main()
