"""Physical constants and NV-centre parameters used by the models.

Same namespace layout as the reference's ``superspinsim/params.py``
(``fundamental``, ``standards.lab.ntp``, ``nv.room.{optical, ground,
excited, isc}``, ``n.n_14``), restricted to the values the generator builder
and the models read.  Values: CODATA (Tiesinga et al., Rev. Mod. Phys. 93,
025010 (2021); Mohr et al., Rev. Mod. Phys. 97, 025002 (2025)) and the NV
room-temperature literature values the reference uses.  ``nv.room.optical``
rates are in 1/s, times in s, frequencies in Hz.
"""


class fundamental:
    planck = 6.62607015e-34
    boltzmann = 1.3806489999999998e-23
    bohr_gyro = 13996244917.1          # Hz/T
    nuclear_gyro = 7622593.2188        # Hz/T
    boltzmann_gyro = 20836619120.0     # Hz/K

    class electron:
        g = 2.00231930436092


class standards:
    class lab:
        class ntp:
            temperature = 293.15
            pressure = 101325.0


class nv:
    class room:
        class optical:
            conserving = 66000000.0
            nonconserving = 3547020.0564265894

        class ground:
            thermalisation_time = 0.01
            dephasing_time = 9.999999999999999e-05
            zfs_longitudinal = 2872000000.0
            g_longitudinal = 2.000536581621305
            g_transverse = 2.0031
            # 14N nuclear spin in the ground state
            thermalisation_time_14N = 10.0
            dephasing_time_14N = 9.999999999999999e-06
            nuclear_quadrupole_14N_longitudinal = -4945000.0
            hyperfine_14N_longitudinal = -2162000.0
            hyperfine_14N_transverse = -2620000.0
            g_N_14N_longitudinal = 0.40366839834155777

        class excited:
            thermalisation_time = 0.001
            dephasing_time = 1e-08
            zfs_longitudinal = 1423000000.0
            g_longitudinal = 2.0019655363224635
            # 14N nuclear spin in the excited state
            thermalisation_time_14N = 0.1
            dephasing_time_14N = 0.001
            nuclear_quadrupole_14N_longitudinal = -4945000.0
            hyperfine_14N_longitudinal = -40000000.0
            hyperfine_14N_transverse = -23000000.0
            g_N_14N_longitudinal = 0.4040619651907696

        class isc:
            s_gets_pm = 60400000.0
            s_gets_z = 9390000.0
            z_gets_s = 9600000.0
            pm_gets_s = 2110000.0


class n:
    class n_14:
        class nmr:
            gyro = -3070000.0
            g = -0.00021934454662776454
