"""sss_simulate_noalloc, the entry point that allocates nothing, against the
plan-based sss_simulate_device on the same device buffers.

It is for callers that cannot allocate device memory (code running inside
another framework's memory pool, a device whose memory is fully reserved,
or a context where allocation is not allowed): its scratch is a fixed
file-scope device array inside libsss.so.  Two calls in a row check that a
call does not depend on what the previous one left in that array; the
first call spans several scratch-sized chunks of output samples."""
import ctypes

import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu


def _bind():
    from superspinsim_gb300 import _lib
    L = _lib.load()
    vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
    i, d = ctypes.c_int, ctypes.c_double
    L.sss_simulate_noalloc.argtypes = [ctypes.POINTER(_lib.PlanDesc), vp, dp, dp, vp, i, i, vp,
                                       d, d, i, i, vp, vp]
    L.sss_simulate_noalloc.restype = i
    return L


def _program(freq, amp, laser):
    p = np.zeros((4, 1, 5))
    p[:, :, 0] = np.inf
    p[0, 0, 2:4] = [amp, freq]
    p[3, 0, 1] = laser
    return p


def test_noalloc_matches_plan_path_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.quadratures import method
    L = _bind()
    c = load_case("nv7_n49")
    gens = np.ascontiguousarray(c["generators"])
    vm = c["vectorisation_map"]
    N = gens.shape[1]
    W, nodes = method(2)
    desc = _lib.PlanDesc(N, 5, 2, 2, _lib.SSS_RESIDUAL, _lib.SSS_EXPM_TAYLOR, 35, 0)
    plan = _lib.Plan(gens, W, nodes)
    d_gens = torch.from_numpy(gens).cuda()
    f_res = 2.870e9 + 28.025e9*5e-3
    calls = [(250, 2, f_res + 2e6, 1), (7, 20, f_res - 9e6, 0)]  # (T, F, drive, ground level)
    for T, F, freq, level in calls:
        rho = np.zeros(N)
        for k, (y, x, ch) in enumerate(vm):
            if y == x == level and ch == 0:
                rho[k] = 1.0
        d_rho0 = torch.from_numpy(rho).cuda()
        d_prog = torch.from_numpy(_program(freq, 5e6/28.025e9, 10/65.9)).cuda()
        out_a = torch.full((T, N), float("nan"), dtype=torch.float64, device="cuda")
        out_b = torch.empty((T, N), dtype=torch.float64, device="cuda")
        dt = 1e-9
        _lib.check(L.sss_simulate_noalloc(
            ctypes.byref(desc), d_gens.data_ptr(), _lib.dptr(W), _lib.dptr(nodes),
            d_rho0.data_ptr(), 4, 1, d_prog.data_ptr(), 0.0, dt, T, F, out_a.data_ptr(), None))
        _lib.check(L.sss_simulate_device(
            plan.handle, 1, d_rho0.data_ptr(), 4, 1, d_prog.data_ptr(), None, 0.0, dt, T, F,
            out_b.data_ptr(), None))
        torch.cuda.synchronize()
        a, b = out_a.cpu().numpy(), out_b.cpu().numpy()
        assert np.isfinite(a).all()
        assert np.abs(a - b).max() <= 1e-12


def test_noalloc_rejects_sizes_beyond_its_limit():
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.quadratures import method
    L = _bind()
    W, nodes = method(2)
    desc = _lib.PlanDesc(53, 5, 2, 2, _lib.SSS_RESIDUAL, _lib.SSS_EXPM_TAYLOR, 35, 0)
    rc = L.sss_simulate_noalloc(ctypes.byref(desc), 1, _lib.dptr(W), _lib.dptr(nodes), 1, 4, 1,
                                1, 0.0, 1e-9, 4, 2, 1, None)
    assert rc == -1
    assert b"N <= 52" in L.sss_last_error()


def _noalloc_vs_plan(L, torch, gens, vm, W, nodes, T, F, freq, level=1):
    """One sss_simulate_noalloc call and the plan path on the same inputs;
    returns the max-abs difference."""
    from superspinsim_gb300 import _lib
    N = gens.shape[1]
    desc = _lib.PlanDesc(N, gens.shape[0], len(W), len(nodes), _lib.SSS_RESIDUAL,
                         _lib.SSS_EXPM_TAYLOR, 35, 0)
    plan = _lib.Plan(gens, W, nodes)
    d_gens = torch.from_numpy(np.ascontiguousarray(gens)).cuda()
    rho = np.zeros(N)
    for k, (y, x, ch) in enumerate(vm):
        if y == x == level and ch == 0:
            rho[k] = 1.0
    d_rho0 = torch.from_numpy(rho).cuda()
    d_prog = torch.from_numpy(_program(freq, 5e6/28.025e9, 10/65.9)).cuda()
    out_a = torch.full((T, N), float("nan"), dtype=torch.float64, device="cuda")
    out_b = torch.empty((T, N), dtype=torch.float64, device="cuda")
    _lib.check(L.sss_simulate_noalloc(
        ctypes.byref(desc), d_gens.data_ptr(), _lib.dptr(W), _lib.dptr(nodes),
        d_rho0.data_ptr(), 4, 1, d_prog.data_ptr(), 0.0, 1e-9, T, F, out_a.data_ptr(), None))
    _lib.check(L.sss_simulate_device(
        plan.handle, 1, d_rho0.data_ptr(), 4, 1, d_prog.data_ptr(), None, 0.0, 1e-9, T, F,
        out_b.data_ptr(), None))
    torch.cuda.synchronize()
    a, b = out_a.cpu().numpy(), out_b.cpu().numpy()
    assert np.isfinite(a).all()
    return float(np.abs(a - b).max())


def test_noalloc_after_a_smaller_plan_run():
    """A plan run at a small N sets the step kernel's shared-memory limit for
    that N; the next large-N noalloc call must still launch."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from superspinsim_gb300.quadratures import method
    L = _bind()
    W, nodes = method(2)
    big, small = load_case("nv7_n49"), load_case("qubit_couple")
    f_res = 2.870e9 + 28.025e9*5e-3
    assert _noalloc_vs_plan(L, torch, big["generators"], big["vectorisation_map"], W, nodes,
                            5, 4, f_res) <= 1e-12
    assert _noalloc_vs_plan(L, torch, small["generators"], small["vectorisation_map"], W, nodes,
                            5, 4, 1e7, level=0) <= 1e-12
    assert _noalloc_vs_plan(L, torch, big["generators"], big["vectorisation_map"], W, nodes,
                            5, 4, f_res - 3e6) <= 1e-12


def test_noalloc_leaves_free_device_memory_unchanged():
    """After a first call, further calls of several lengths take no device
    memory (the free bytes the driver reports do not move)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from superspinsim_gb300 import _lib
    from superspinsim_gb300.quadratures import method
    L = _bind()
    c = load_case("nv7_n49")
    gens = np.ascontiguousarray(c["generators"])
    N = gens.shape[1]
    W, nodes = method(2)
    desc = _lib.PlanDesc(N, 5, 2, 2, _lib.SSS_RESIDUAL, _lib.SSS_EXPM_TAYLOR, 35, 0)
    d_gens = torch.from_numpy(gens).cuda()
    rho = np.zeros(N)
    rho[1] = 1.0
    d_rho0 = torch.from_numpy(rho).cuda()
    d_prog = torch.from_numpy(_program(2.870e9 + 28.025e9*5e-3, 5e6/28.025e9, 10/65.9)).cuda()
    out = torch.empty((300, N), dtype=torch.float64, device="cuda")

    def call(T):
        _lib.check(L.sss_simulate_noalloc(
            ctypes.byref(desc), d_gens.data_ptr(), _lib.dptr(W), _lib.dptr(nodes),
            d_rho0.data_ptr(), 4, 1, d_prog.data_ptr(), 0.0, 1e-9, T, 2, out.data_ptr(), None))
        torch.cuda.synchronize()

    call(3)
    free0 = torch.cuda.mem_get_info()[0]
    for T in (1, 40, 300, 7):
        call(T)
    assert torch.cuda.mem_get_info()[0] == free0
    assert np.isfinite(out.cpu().numpy()).all()
