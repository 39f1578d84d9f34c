"""The allocation-free mode-to-mode entry point (fit_mode_to_mode_noalloc) against fit_mode_to_mode.

Callers that cannot allocate device memory (a caller-owned memory budget or allocator, a
latency-critical loop, an embedding runtime lending only its own buffers) use the no-allocation
variant; it must give the same S(k|p) and net(k) as the allocating entry point, on consecutive
calls that reuse its fixed scratch array. FP64 products: within 1e-12 relative (max-norm);
FP32 products: within 1e-5 relative. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import fit_gb300 as F
from fields import curl_noise_3d, solenoidal_2d

pytestmark = pytest.mark.gpu


def _entry():
    lib = F._lib.load()
    fn = lib.fit_mode_to_mode_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.POINTER(C.c_int64), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p), C.c_int,
                   C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return lib, fn


def _dev(a):
    import torch
    raw = np.ascontiguousarray(np.asarray(a).ravel(order="F").view(np.float64))
    return torch.from_numpy(raw).cuda()


@pytest.mark.parametrize("case", ["2d", "3d_helicity"])
@pytest.mark.parametrize("fp64", [True, False])
def test_no_alloc_matches_allocating_entry(case, fp64):
    import torch
    lib, fn = _entry()
    if case == "2d":
        u, ks = solenoidal_2d(12, 21)
        inv, code = F.KineticEnergy(), 0
    else:
        u, ks = curl_noise_3d(8, 7)
        inv, code = F.Helicity(), 2
    nd = len(ks)
    ns = u.shape[:nd]
    nm = int(np.prod(ns))
    ref = F.calculate_mode_to_mode_transfer(u, ks, invariant=inv, force=True, fp64_products=fp64)
    u_d = _dev(np.asfortranarray(u.astype(np.complex128)))
    ks_d = [torch.tensor(np.asarray(k, dtype=np.float64), device="cuda") for k in ks]
    ks_arr = (C.c_void_p * nd)(*[k.data_ptr() for k in ks_d])
    nsv = (C.c_int64 * nd)(*ns)
    tol = 1e-12 if fp64 else 1e-5
    S_ref = np.asarray(ref.transfer, dtype=np.float64).ravel(order="F")
    net_ref = np.asarray(ref.net_transfer, dtype=np.float64).ravel(order="F")
    for _ in range(2):                       # two calls in a row share the scratch array
        S = torch.full((nm * nm,), float("nan"), dtype=torch.float64, device="cuda")
        net = torch.full((nm,), float("nan"), dtype=torch.float64, device="cuda")
        rc = fn(nd, nsv, u.shape[nd], u.shape[nd], 1, ks_arr, code, int(fp64), 1, C.c_void_p(u_d.data_ptr()), None,
                C.c_void_p(S.data_ptr()), C.c_void_p(net.data_ptr()), None)
        assert rc == 0, lib.fit_last_error()
        got = S.cpu().numpy()
        assert np.max(np.abs(got - S_ref)) <= tol * 10 * np.max(np.abs(S_ref))
        assert np.max(np.abs(net.cpu().numpy() - net_ref)) <= tol * 100 * np.max(np.abs(S_ref))


def test_no_alloc_rejects_grids_above_the_limit():
    lib, fn = _entry()
    nsv = (C.c_int64 * 3)(64, 64, 64)
    ks_arr = (C.c_void_p * 3)(None, None, None)
    rc = fn(3, nsv, 3, 3, 1, ks_arr, 0, 1, 1, C.c_void_p(16), None, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == -2 and b"32768" in lib.fit_last_error()
