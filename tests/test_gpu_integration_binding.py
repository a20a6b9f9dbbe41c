"""The reference-side binding of the integration notes: plain ctypes on
libsss.so (no package helpers), as a maintainer of the reference would add
it -- sss_simulate with a host-sampled coefficient table, sss_batch_run for
a sweep of programs and sss_batch_run_table for the same sweep from sampled
rows -- against the oracle."""
import ctypes

import numpy as np
import pytest

from conftest import load_case, quadrature
from oracle import oracle

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class _Desc(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("G", ctypes.c_int), ("K", ctypes.c_int),
                ("Q", ctypes.c_int), ("flags", ctypes.c_uint), ("expm", ctypes.c_int),
                ("quartic_repeats", ctypes.c_int), ("taylor_degree", ctypes.c_int)]


def _bind():
    from superspinsim_gb300 import build
    lib = ctypes.CDLL(build.build())
    lib.sss_plan_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(_Desc),
                                    _dp, _dp, _dp]
    lib.sss_simulate.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int,
                                 _dp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                 ctypes.c_int, _dp, ctypes.c_void_p]
    lib.sss_batch_run.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int,
                                  _dp, _ip, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int, ctypes.c_void_p]
    lib.sss_batch_run_table.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _ip,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int,
                                        ctypes.c_void_p]
    lib.sss_last_error.restype = ctypes.c_char_p
    lib.sss_plan_destroy.argtypes = [ctypes.c_void_p]
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def test_reference_side_ctypes_binding():
    lib = _bind()

    def check(rc):
        assert rc == 0, lib.sss_last_error().decode()

    c = load_case("nv7_n49")
    gens, vm = np.ascontiguousarray(c["generators"]), c["vectorisation_map"]
    G, N, _ = gens.shape
    W, nodes = quadrature(2)
    K, Q = W.shape
    plan = ctypes.c_void_p()
    d = _Desc(N, G, K, Q, 1, 0, 35, 0)    # residual, the reference's exponential
    check(lib.sss_plan_create(ctypes.byref(plan), ctypes.byref(d), _p(gens),
                              _p(np.ascontiguousarray(W)), _p(np.ascontiguousarray(nodes))))
    try:
        f_res = 2.870e9 + 28.025e9*5e-3
        amp, laser = 5e6/28.025e9, 10/65.9
        rho = np.zeros((7, 7), complex)
        rho[1, 1] = 1
        flat0 = oracle.flatten(rho, vm, N)
        T, dt, F = 3, 1e-9, 20
        # sss_simulate with the coefficient table a reference sampler writes:
        # row (r*T + t)*Q + k holds [1, x, y, z, laser] at the node time
        tab = np.zeros((F*T*Q, G))
        for r in range(F):
            for t in range(T):
                for k in range(Q):
                    tn = ((0.0 + (r*dt)/F) + dt*t) + (dt*nodes[k])/F
                    tab[(r*T + t)*Q + k] = [1.0, amp*np.cos(2*np.pi*f_res*tn), 0, 0, laser]
        out = np.empty((T, N))
        check(lib.sss_simulate(plan, 1, _p(np.ascontiguousarray(flat0)), 0, 1, None, _p(tab),
                               0.0, dt, T, F, _p(out), None))
        prog = np.zeros((4, 1, 5))
        prog[:, :, 0] = np.inf
        prog[0, 0, 2], prog[0, 0, 3], prog[3, 0, 1] = amp, f_res, laser
        _, ref = oracle.simulate(gens, rho, 0.0, T*dt + 1e-13, dt, prog, K=2, W=W, nodes=nodes,
                                 F=F, vectorisation_map=vm, flat_out=True)
        assert np.abs(out - ref).max() <= 1e-12
        # sss_batch_run: a sweep over four drive frequencies
        freqs = f_res + np.array([-2e6, 0.0, 1e6, 3e6])
        progs = np.repeat(prog[None], 4, axis=0)
        progs[:, 0, 0, 3] = freqs
        rho0 = np.repeat(flat0[None], 4, axis=0)
        w = np.array([1.0 if (y == x and y in (3, 4, 5) and cc == 0) else 0.0
                      for y, x, cc in vm])
        ro, fin = np.empty((4, T)), np.empty((4, N))
        check(lib.sss_batch_run(plan, 4, _p(rho0), 4, 1, _p(np.ascontiguousarray(progs)), None,
                                0.0, dt, T, F, _p(w), _p(ro), _p(fin), None, 1, None))
        _, refb = oracle.simulate(gens, np.stack([rho]*4), 0.0, T*dt + 1e-13, dt, progs, K=2,
                                  W=W, nodes=nodes, F=F, vectorisation_map=vm, mode="vector",
                                  degree=16, flat_out=True)
        assert np.abs(fin - refb[:, -1]).max() <= 1e-12
        assert np.abs(ro - refb @ w).max() <= 1e-12
        # sss_batch_run_table: the same sweep from sampled rows (a sampler
        # callable per trajectory), as the integration notes bind it
        tabs = np.zeros((4, F*T*Q, G))
        for b, f in enumerate(freqs):
            for r in range(F):
                for t in range(T):
                    for k in range(Q):
                        tn = ((0.0 + (r*dt)/F) + dt*t) + (dt*nodes[k])/F
                        tabs[b, (r*T + t)*Q + k] = [1.0, amp*np.cos(2*np.pi*f*tn), 0, 0, laser]
        ro2, fin2 = np.empty((4, T)), np.empty((4, N))
        check(lib.sss_batch_run_table(plan, 4, _p(rho0), _p(tabs), None, 0.0, dt, T, F, _p(w),
                                      _p(ro2), _p(fin2), None, 1, None))
        assert np.abs(fin2 - refb[:, -1]).max() <= 1e-12
        assert np.abs(ro2 - refb @ w).max() <= 1e-12
    finally:
        lib.sss_plan_destroy(plan)
