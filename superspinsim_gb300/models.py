"""Ready-made spin descriptions (reference ``superspinsim/models.py``).

``nv_7`` returns the reference's 7-level NV description (ground and excited
spin-1 triplets and the metastable singlet, with optical and intersystem
crossing couplings), in the same format, for ``generate_atoms`` /
``simspins``.  ``odmr_params`` is the parameter set of the 7-level ODMR
workload (rates overridden, see its docstring).
"""
import math
import types

import numpy as np

from superspinsim_gb300 import params as s3p


def nv_7(quiescent_magnetic_field=None, params=None):
    """(spins, spin_interactions, group_interactions) of the 7-level NV
    (reference models.py:9-87): levels g+, g0, g-, e+, e0, e-, s."""
    B0 = np.zeros(3) if quiescent_magnetic_field is None else np.asarray(
        quiescent_magnetic_field, dtype=float)
    P = s3p if params is None else params
    ground = {"S": 1, "g": P.nv.room.ground.g_longitudinal,
              "g_perp": P.nv.room.ground.g_transverse,
              "D": math.tau*P.nv.room.ground.zfs_longitudinal,
              "TS1": P.nv.room.ground.thermalisation_time,
              "TS2": P.nv.room.ground.dephasing_time,
              "B0": B0, "T": P.standards.lab.ntp.temperature}
    excited = {"S": 1, "g": P.nv.room.excited.g_longitudinal,
               "D": math.tau*P.nv.room.excited.zfs_longitudinal,
               "TS1": P.nv.room.excited.thermalisation_time,
               "TS2": P.nv.room.excited.dephasing_time,
               "B0": B0, "T": P.standards.lab.ntp.temperature}
    singlet = {"S": 0}
    groups = {
        ((0, 0), (1, 0)): {"rel": P.nv.room.optical.conserving,
                           "rel_n": P.nv.room.optical.nonconserving},
        ((1, 0), (2, 0)): {"s_gets_0": P.nv.room.isc.s_gets_z,
                           "s_gets_1": P.nv.room.isc.s_gets_pm},
        ((2, 0), (0, 0)): {"0_gets_s": P.nv.room.isc.z_gets_s,
                           "1_gets_s": P.nv.room.isc.pm_gets_s},
    }
    return [[ground], [excited], [singlet]], [{}, {}, {}], groups


def odmr_params():
    """Parameters of the 7-level ODMR workload: ground D = 2.870 GHz,
    excited D = 1.42 GHz, spin-conserving optical decay 65.9 /us only,
    ISC 11 /us (ms=0) and 80 /us (ms=+-1) into the singlet, singlet decay
    3.0 /us to ms=0 and 2.6 /us to ms=+-1; everything else as ``params``."""
    P = types.SimpleNamespace(fundamental=s3p.fundamental, standards=s3p.standards)

    class ground(s3p.nv.room.ground):
        zfs_longitudinal = 2.870e9

    class excited(s3p.nv.room.excited):
        zfs_longitudinal = 1.42e9

    class optical(s3p.nv.room.optical):
        conserving = 65.9e6
        nonconserving = None

    class isc(s3p.nv.room.isc):
        s_gets_z = 11e6
        s_gets_pm = 80e6
        z_gets_s = 3.0e6
        pm_gets_s = 2.6e6

    room = types.SimpleNamespace(ground=ground, excited=excited, optical=optical, isc=isc)
    P.nv = types.SimpleNamespace(room=room)
    return P


def nv_21(quiescent_magnetic_field=None, params=None):
    """The 21-level NV with its 14N nucleus (spin 1) in every orbital
    manifold: the description the reference's legacy ``generate_21``
    builds (superspinsim/generate_generators.py:2944-3028), returned in the
    ``nv_7`` format for ``generate_atoms`` / ``simspins``."""
    B0 = np.zeros(3) if quiescent_magnetic_field is None else np.asarray(
        quiescent_magnetic_field, dtype=float)
    P = s3p if params is None else params
    g, e = P.nv.room.ground, P.nv.room.excited
    T = P.standards.lab.ntp.temperature
    ground = {"S": 1, "g": g.g_longitudinal, "g_perp": g.g_transverse,
              "D": math.tau*g.zfs_longitudinal, "TS1": g.thermalisation_time,
              "TS2": g.dephasing_time,
              "I": 1, "gN": g.g_N_14N_longitudinal,
              "P": math.tau*g.nuclear_quadrupole_14N_longitudinal,
              "TI1": g.thermalisation_time_14N, "TI2": g.dephasing_time_14N,
              "A": math.tau*g.hyperfine_14N_longitudinal,
              "A_perp": math.tau*g.hyperfine_14N_transverse,
              "B0": B0, "T": T}
    excited = {"S": 1, "g": e.g_longitudinal, "D": math.tau*e.zfs_longitudinal,
               "TS1": e.thermalisation_time, "TS2": e.dephasing_time,
               "I": 1, "gN": e.g_N_14N_longitudinal,
               "P": math.tau*e.nuclear_quadrupole_14N_longitudinal,
               "TI1": e.thermalisation_time_14N, "TI2": e.dephasing_time_14N,
               "A": math.tau*e.hyperfine_14N_longitudinal,
               "A_perp": math.tau*e.hyperfine_14N_transverse,
               "B0": B0, "T": T}
    singlet = {"S": 0, "I": 1, "gN": g.g_N_14N_longitudinal,
               "P": math.tau*g.nuclear_quadrupole_14N_longitudinal,
               "TI1": g.thermalisation_time_14N, "TI2": g.dephasing_time_14N,
               "B0": B0, "T": T}
    _, _, groups = nv_7(B0, params)
    return [[ground], [excited], [singlet]], [{}, {}, {}], groups


def nv21_params():
    """The dense 21-level workload's parameters: the 7-level ODMR rates
    (``odmr_params``) with the ground-state 14N hyperfine A_par = -2.16 MHz,
    A_perp = -2.70 MHz and quadrupole P = -4.95 MHz."""
    P = odmr_params()

    class ground(P.nv.room.ground):
        hyperfine_14N_longitudinal = -2.16e6
        hyperfine_14N_transverse = -2.70e6
        nuclear_quadrupole_14N_longitudinal = -4.95e6

    room = types.SimpleNamespace(ground=ground, excited=P.nv.room.excited,
                                 optical=P.nv.room.optical, isc=P.nv.room.isc)
    P.nv = types.SimpleNamespace(room=room)
    return P
