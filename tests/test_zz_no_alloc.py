"""The allocation-free mode-to-mode entry point (fit_mode_to_mode_noalloc) against fit_mode_to_mode.

Callers that cannot allocate device memory (a caller-owned memory budget or allocator, a
latency-critical loop, an embedding runtime lending only its own buffers) use the no-allocation
variant; it must give the same S(k|p) and net(k) as the allocating entry point, on consecutive
calls that reuse its fixed scratch array. FP64 products: within 1e-12 relative (max-norm);
FP32 products: within 1e-5 relative. Cases: ComplexF64 and ComplexF32 inputs, NoDealiasing and
the 2/3 rule, a passive scalar advected by a separate velocity, a 32^3 three-component grid
at the 32768-mode limit, where the scratch layout is fullest, and a call captured into a CUDA
graph and replayed. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import fit_gb300 as F
from fields import curl_noise_3d, e_config2, scalar_2d, solenoidal_2d, spectrum_field

pytestmark = pytest.mark.gpu


def _entry():
    lib = F._lib.load()
    fn = lib.fit_mode_to_mode_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.POINTER(C.c_int64), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p), C.c_int,
                   C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return lib, fn


def _dev(a, io64=True):
    """Column-major complex field on the device as interleaved floats of the io precision."""
    import torch
    a = np.asarray(a, dtype=np.complex128 if io64 else np.complex64)
    raw = np.ascontiguousarray(a.ravel(order="F").view(np.float64 if io64 else np.float32))
    return torch.from_numpy(raw).cuda()


def _ks_dev(ks):
    import torch
    ks_d = [torch.tensor(np.asarray(k, dtype=np.float64), device="cuda") for k in ks]
    return ks_d, (C.c_void_p * len(ks))(*[k.data_ptr() for k in ks_d])


CASES = {
    "2d_ke": lambda: (*solenoidal_2d(12, 21), None, F.KineticEnergy(), 0),
    "3d_helicity": lambda: (*curl_noise_3d(8, 7), None, F.Helicity(), 2),
    "2d_scalar": lambda: (scalar_2d(12, 5), solenoidal_2d(12, 6)[1], solenoidal_2d(12, 6)[0], F.PassiveScalar(), 1),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("fp64", [True, False])
@pytest.mark.parametrize("io64", [True, False])
@pytest.mark.parametrize("dealias", [0, 1])
def test_no_alloc_matches_allocating_entry(case, fp64, io64, dealias):
    import torch
    lib, fn = _entry()
    u, ks, adv, inv, code = CASES[case]()
    cdt = np.complex128 if io64 else np.complex64
    u = np.asfortranarray(u.astype(cdt))
    adv = None if adv is None else np.asfortranarray(adv.astype(cdt))
    nd = len(ks)
    ns = u.shape[:nd]
    nm = int(np.prod(ns))
    dl = F.OrszagTwoThirds() if dealias else F.NoDealiasing()
    # the allocating entry's FP64 outputs (the public function rounds them to the input's precision)
    plan = F.api._plan(u, ks, dl, F.GB300Spectral(), adv)
    S_all, net_all = plan.mode_to_mode(u, inv.code, fp64, adv)
    u_d = _dev(u, io64)
    a_d = None if adv is None else _dev(adv, io64)
    ks_d, ks_arr = _ks_dev(ks)
    nsv = (C.c_int64 * nd)(*ns)
    tol = 1e-12 if fp64 else 1e-5
    S_ref = np.asarray(S_all, dtype=np.float64).ravel(order="F")
    net_ref = np.asarray(net_all, dtype=np.float64).ravel(order="F")
    D = u.shape[nd] if adv is None else adv.shape[nd]
    for _ in range(2):                       # two calls in a row share the scratch array
        S = torch.full((nm * nm,), float("nan"), dtype=torch.float64, device="cuda")
        net = torch.full((nm,), float("nan"), dtype=torch.float64, device="cuda")
        rc = fn(nd, nsv, u.shape[nd], D, dealias, ks_arr, code, int(fp64), int(io64), C.c_void_p(u_d.data_ptr()),
                None if a_d is None else C.c_void_p(a_d.data_ptr()), C.c_void_p(S.data_ptr()),
                C.c_void_p(net.data_ptr()), None)
        assert rc == 0, lib.fit_last_error()
        got = S.cpu().numpy()
        scale = np.max(np.abs(S_ref))
        assert np.max(np.abs(got - S_ref)) <= tol * 10 * scale
        assert np.max(np.abs(net.cpu().numpy() - net_ref)) <= tol * 100 * scale


def test_no_alloc_at_the_mode_limit():
    """32^3 three-component field (32768 modes, the fixed limit; S is 8.6 GB): both entry points
    write S on the device; FP64 products within 1e-12 of max|S|, on two calls in a row."""
    import torch
    lib, fn = _entry()
    u, ks = spectrum_field((32, 32, 32), e_config2, seed=8)
    nm = 32 ** 3
    u_d = _dev(u)
    ks_d, ks_arr = _ks_dev(ks)
    nsv = (C.c_int64 * 3)(32, 32, 32)
    plan = F.plan.get_plan((32, 32, 32), 3, 3, "two_thirds", 64, True, ks)
    S_ref = torch.empty(nm * nm, dtype=torch.float64, device="cuda")
    net_ref = torch.empty(nm, dtype=torch.float64, device="cuda")
    F._lib.check(lib.fit_mode_to_mode(plan.h, C.c_void_p(u_d.data_ptr()), None, 0, 1, C.c_void_p(S_ref.data_ptr()),
                                      C.c_void_p(net_ref.data_ptr()), F._lib.PTR_DEVICE))
    scale = float(S_ref.abs().max())
    S = torch.empty_like(S_ref)
    net = torch.empty_like(net_ref)
    for _ in range(2):
        S.fill_(float("nan"))
        net.fill_(float("nan"))
        rc = fn(3, nsv, 3, 3, 1, ks_arr, 0, 1, 1, C.c_void_p(u_d.data_ptr()), None, C.c_void_p(S.data_ptr()),
                C.c_void_p(net.data_ptr()), None)
        assert rc == 0, lib.fit_last_error()
        assert float((S - S_ref).abs().max()) <= 1e-12 * scale
        assert float((net - net_ref).abs().max()) <= 1e-10 * scale
    del S, S_ref
    torch.cuda.empty_cache()


def test_no_alloc_captured_in_a_cuda_graph():
    """After one eager call, a call on a stream under capture enqueues its kernels without
    synchronising (the capture stays valid); replaying the graph reproduces the eager S and net."""
    import torch
    lib, fn = _entry()
    u, ks = curl_noise_3d(8, 7)
    u = np.asfortranarray(u.astype(np.complex128))
    nm = 8 ** 3
    u_d = _dev(u)
    ks_d, ks_arr = _ks_dev(ks)
    nsv = (C.c_int64 * 3)(8, 8, 8)
    S = torch.full((nm * nm,), float("nan"), dtype=torch.float64, device="cuda")
    net = torch.full((nm,), float("nan"), dtype=torch.float64, device="cuda")
    args = (3, nsv, 3, 3, 1, ks_arr, 2, 1, 1, C.c_void_p(u_d.data_ptr()), None, C.c_void_p(S.data_ptr()),
            C.c_void_p(net.data_ptr()))
    assert fn(*args, None) == 0, lib.fit_last_error()
    S_ref, net_ref = S.clone(), net.clone()
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
        rc = fn(*args, C.c_void_p(side.cuda_stream))
    assert rc == 0, lib.fit_last_error()
    S.fill_(float("nan"))
    net.fill_(float("nan"))
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    scale = float(S_ref.abs().max())
    assert float((S - S_ref).abs().max()) <= 1e-14 * scale
    assert float((net - net_ref).abs().max()) <= 1e-12 * scale


def test_no_alloc_rejects_grids_above_the_limit():
    lib, fn = _entry()
    nsv = (C.c_int64 * 3)(64, 64, 64)
    ks_arr = (C.c_void_p * 3)(None, None, None)
    rc = fn(3, nsv, 3, 3, 1, ks_arr, 0, 1, 1, C.c_void_p(16), None, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == -2 and b"32768" in lib.fit_last_error()


def test_no_alloc_rejects_host_and_null_pointers():
    """A NULL wavenumber table or a host array is an argument error, returned before any launch."""
    import torch
    lib, fn = _entry()
    u, ks = solenoidal_2d(8, 3)
    u_d = _dev(u)
    ks_d, ks_arr = _ks_dev(ks)
    nsv = (C.c_int64 * 2)(8, 8)
    S = torch.empty(64 * 64, dtype=torch.float64, device="cuda")
    net = torch.empty(64, dtype=torch.float64, device="cuda")
    before = F.launch_count()
    null_ks = (C.c_void_p * 2)(ks_arr[0], None)
    rc = fn(2, nsv, 2, 2, 1, null_ks, 0, 1, 1, C.c_void_p(u_d.data_ptr()), None, C.c_void_p(S.data_ptr()),
            C.c_void_p(net.data_ptr()), None)
    assert rc == -1 and b"ks_dev[1]" in lib.fit_last_error()
    host_u = np.ascontiguousarray(u.ravel(order="F"))
    rc = fn(2, nsv, 2, 2, 1, ks_arr, 0, 1, 1, C.c_void_p(host_u.ctypes.data), None, C.c_void_p(S.data_ptr()),
            C.c_void_p(net.data_ptr()), None)
    assert rc == -1 and b"u_hat" in lib.fit_last_error()
    host_S = np.empty(64 * 64)
    rc = fn(2, nsv, 2, 2, 1, ks_arr, 0, 1, 1, C.c_void_p(u_d.data_ptr()), None, C.c_void_p(host_S.ctypes.data),
            C.c_void_p(net.data_ptr()), None)
    assert rc == -1 and b"S must" in lib.fit_last_error()
    assert F.launch_count() == before
