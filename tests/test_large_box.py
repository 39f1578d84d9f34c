"""The live-box FP32 forms at full size (512^3, transform length 512) against the plans' FP64 paths on
the same device field: one-pass partial fluxes of kinetic energy and helicity, smooth band-to-band,
and the spectral flux. Device pointers throughout; fields are seeded complex-normal noise (the box
forms take the Hermitian part, as the FP64 paths do)."""
import numpy as np
import pytest

import fit_gb300 as F

pytestmark = pytest.mark.gpu

N = 512


def _setup():
    torch = pytest.importorskip("torch")
    F.clear_plans()
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(21)
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = torch.randn((3, N, N, N), device=dev, dtype=torch.complex64, generator=g)
    return torch, dev, ns, ks, u


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_partial_fluxes_box_512():
    torch, dev, ns, ks, u = _setup()
    edges = np.asarray(F.shell_edges(F.DyadicBinning(1.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    invs = [F.KineticEnergy().code, F.Helicity().code]
    p32 = F.Plan(ns, 3, 3, "two_thirds", 32, False, ks)
    T = torch.zeros(2 * 8 * nsh, dtype=torch.float64, device=dev)
    p32.partial_fluxes_batched_device(u.data_ptr(), 1, invs, edges, 7, False, T.data_ptr())
    torch.cuda.synchronize()
    T32 = T.cpu().numpy().reshape(2, 8, nsh)
    del p32
    F.clear_plans()
    u64 = u.to(torch.complex128)
    p64 = F.Plan(ns, 3, 3, "two_thirds", 64, True, ks)
    Tq = torch.zeros(8 * nsh, dtype=torch.float64, device=dev)
    for j, inv in enumerate(invs):
        p64.partial_fluxes_device(u64.data_ptr(), 1, inv, edges, 7, False, Tq.data_ptr())
        torch.cuda.synchronize()
        assert _rel(T32[j], Tq.cpu().numpy().reshape(8, nsh)) < 1e-5, inv


def test_band_to_band_box_512():
    torch, dev, ns, ks, u = _setup()
    centers = [2.0 ** j for j in range(1, 8)]
    nb = len(centers)
    out = {}
    for prec, field in ((32, u), (64, u.to(torch.complex128))):
        plan = F.Plan(ns, 3, 3, "two_thirds", prec, prec == 64, ks)
        T = torch.zeros((nb, nb), dtype=torch.float64, device=dev)
        plan.band_to_band_device(field.data_ptr(), 0, centers, 0.6, 7, False, F.KineticEnergy().code, T.data_ptr(),
                                 0, 0)
        torch.cuda.synchronize()
        out[prec] = T.cpu().numpy()
        del plan
        F.clear_plans()
    assert np.max(np.abs(out[64])) > 0
    assert _rel(out[32], out[64]) < 1e-5


def test_spectral_flux_box_512():
    torch, dev, ns, ks, u = _setup()
    edges = np.asarray(F.shell_edges(F.LinearBinning(14.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    out = {}
    for prec, field in ((32, u), (64, u.to(torch.complex128))):
        plan = F.Plan(ns, 3, 3, "two_thirds", prec, prec == 64, ks)
        T = torch.zeros(nsh, dtype=torch.float64, device=dev)
        P = torch.zeros(nsh, dtype=torch.float64, device=dev)
        plan.spectral_flux_device(field.data_ptr(), 0, 0, edges, 7, False, F.Helicity().code, T.data_ptr(),
                                  P.data_ptr())
        torch.cuda.synchronize()
        out[prec] = (T.cpu().numpy(), P.cpu().numpy())
        del plan
        F.clear_plans()
    assert _rel(out[32][0], out[64][0]) < 1e-5
    assert _rel(out[32][1], out[64][1]) < 1e-5
