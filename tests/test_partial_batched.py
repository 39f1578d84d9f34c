"""One-pass, graph-replayed partial fluxes of several invariants (fit_partial_fluxes_batched)
against the oracle's per-invariant partial fluxes (src/SpectralFlux.jl:240-285)."""
import numpy as np
import pytest

import oracle as O
from fields import curl_noise_3d, solenoidal_2d

import fit_gb300 as F

pytestmark = pytest.mark.gpu

DEAL = {"two_thirds": F.OrszagTwoThirds(), "three_halves": F.PaddedThreeHalves(), "none": F.NoDealiasing()}
TOL = {64: 1e-11, 32: 1e-4}


def _check(res, u, ks, decomposition, deal, invs, prec):
    for inv, oinv in invs:
        chans, _, _ = O.partial_fluxes(u, ks, decomposition, ("linear", 1.0), deal, invariant=oinv)
        scale = max(np.max(np.abs(c[0])) for c in chans.values())
        r = res[type(inv).__name__]
        for key, (T, _) in chans.items():
            assert np.max(np.abs(r.channels[key].transfer_spectrum - T)) <= TOL[prec] * scale, (oinv, key)


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("deal", ["two_thirds", "three_halves"])
def test_helical_ke_and_helicity_one_pass(prec, deal):
    u, ks = curl_noise_3d(12, 91)
    invs = ((F.KineticEnergy(), "ke"), (F.Helicity(), "helicity"))
    runs = []
    for _ in range(3):   # eager, capture + launch, replay
        runs.append(F.calculate_partial_fluxes_multi(u, ks, invariants=[i for i, _ in invs],
                                                     binning=F.LinearBinning(1.0), dealiasing=DEAL[deal],
                                                     spectral=F.GB300Spectral(prec)))
    _check(runs[-1], u, ks, "helical", deal, invs, prec)
    for name in ("KineticEnergy", "Helicity"):
        for key, c in runs[0][name].channels.items():
            ref = c.transfer_spectrum
            for r in runs[1:]:
                assert np.max(np.abs(r[name].channels[key].transfer_spectrum - ref)) <= 1e-12 * max(
                    np.max(np.abs(ref)), 1e-300)


def test_helmholtz_ke_and_enstrophy_one_pass():
    u, ks = solenoidal_2d(16, 92)
    rng = np.random.default_rng(0)
    u = u + 0.3 * np.fft.fftn(rng.standard_normal((16, 16, 2)), axes=(0, 1)) / 256   # add a divergent part
    invs = ((F.KineticEnergy(), "ke"), (F.Enstrophy(), "enstrophy"))
    res = F.calculate_partial_fluxes_multi(u, ks, invariants=[i for i, _ in invs],
                                           decomposition=F.HelmholtzDecomposition(), binning=F.LinearBinning(1.0),
                                           spectral=F.GB300Spectral(64))
    _check(res, u, ks, "helmholtz", "two_thirds", invs, 64)


def test_batched_execution_matches_plain():
    u, ks = curl_noise_3d(16, 5)
    a = F.calculate_partial_fluxes(u, ks, binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(64),
                                   invariant=F.Helicity())
    b = F.calculate_partial_fluxes(u, ks, binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(64),
                                   invariant=F.Helicity(), execution=F.GB300Execution("batched"))
    for key, c in a.channels.items():
        assert np.max(np.abs(b.channels[key].transfer_spectrum - c.transfer_spectrum)) <= 1e-12 * max(
            np.max(np.abs(c.transfer_spectrum)), 1e-300)


def test_device_path_replays():
    import torch
    u, ks = curl_noise_3d(16, 7)
    ns = u.shape[:3]
    ud = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(u).ravel(order="F"))).cuda()
    edges = np.asarray(F.shell_edges(F.LinearBinning(1.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    T = torch.zeros(2 * 8 * nsh, dtype=torch.float64, device="cuda")
    p = F.Plan(ns, 3, 3, "two_thirds", 32, True, ks)
    l0 = F.launch_count()
    for _ in range(3):
        p.partial_fluxes_batched_device(ud.data_ptr(), 1, [0, 2], edges, 7, False, T.data_ptr())
    torch.cuda.synchronize()
    assert F.launch_count() > l0
    got = T.cpu().numpy().reshape(2, 8, nsh)
    chans, _, _ = O.partial_fluxes(u, ks, "helical", ("linear", 1.0), "two_thirds", invariant="helicity")
    names = ("positive", "negative")
    scale = max(np.max(np.abs(c[0])) for c in chans.values())
    for sk in range(2):
        for sp in range(2):
            for sq in range(2):
                ref = chans[(names[sk], names[sp], names[sq])][0]
                assert np.max(np.abs(got[1, sk * 4 + sp * 2 + sq] - ref)) <= 1e-4 * scale


def test_errors():
    u, ks = solenoidal_2d(16, 1)
    with pytest.raises(ValueError):
        F.calculate_partial_fluxes_multi(u, ks, invariants=[F.KineticEnergy()])   # helical needs 3D
    u3, ks3 = curl_noise_3d(8, 1)
    with pytest.raises(ValueError):
        F.calculate_partial_fluxes_multi(u3, ks3, invariants=[F.PassiveScalar()])


@pytest.mark.parametrize("deal", ["two_thirds", "three_halves"])
def test_live_box_form_64(deal):
    """FP32 cubic plans of a fused transform size take the live-box form (the four terms as one
    batch of whole-box passes, one binning pass); against the oracle, eager, captured and replayed.
    (The Helmholtz split is 2D-only, as in the reference, so only the helical form reaches it.)"""
    u, ks = curl_noise_3d(64, 13)
    invs = ((F.KineticEnergy(), "ke"), (F.Helicity(), "helicity"))
    runs = []
    for _ in range(3):
        runs.append(F.calculate_partial_fluxes_multi(u, ks, invariants=[i for i, _ in invs],
                                                     binning=F.LinearBinning(1.0), dealiasing=DEAL[deal],
                                                     spectral=F.GB300Spectral(32)))
    _check(runs[-1], u, ks, "helical", deal, invs, 32)
    for name in runs[0]:
        for key, c in runs[0][name].channels.items():
            assert np.array_equal(runs[2][name].channels[key].transfer_spectrum, c.transfer_spectrum)


@pytest.mark.parametrize("prec", [64, 32])
def test_toroidal_poloidal_split_and_partial_fluxes(prec):
    """ToroidalPoloidalDecomposition (src/Decomposition.jl:107-141) on the GPU against the oracle: the
    split itself, the per-invariant partial fluxes and the one-pass form (eager, replayed)."""
    u, ks = curl_noise_3d(16, 57)
    d = F.decompose_field(F.ToroidalPoloidalDecomposition(), u, ks)
    o = O.toroidal_poloidal_decompose(u, ks)
    for name in ("toroidal", "poloidal"):
        assert np.max(np.abs(d[name] - o[name])) <= 1e-12 * np.max(np.abs(o[name]))
    v = u.astype(np.complex64) if prec == 32 else u
    r = F.calculate_partial_fluxes(v, ks, decomposition=F.ToroidalPoloidalDecomposition(),
                                   binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(prec))
    _check({"KineticEnergy": r}, u, ks, "toroidal_poloidal", "two_thirds", ((F.KineticEnergy(), "ke"),), prec)
    invs = ((F.KineticEnergy(), "ke"), (F.Helicity(), "helicity"))
    for _ in range(2):
        m = F.calculate_partial_fluxes_multi(v, ks, invariants=[i for i, _ in invs],
                                             decomposition=F.ToroidalPoloidalDecomposition(),
                                             binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(prec))
    _check(m, u, ks, "toroidal_poloidal", "two_thirds", invs, prec)


def test_toroidal_poloidal_live_box_64():
    """The toroidal/poloidal split on the live-box partial-flux form (FP32, 64^3)."""
    u, ks = curl_noise_3d(64, 59)
    invs = ((F.KineticEnergy(), "ke"), (F.Helicity(), "helicity"))
    m = F.calculate_partial_fluxes_multi(u, ks, invariants=[i for i, _ in invs],
                                         decomposition=F.ToroidalPoloidalDecomposition(),
                                         binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(32))
    _check(m, u, ks, "toroidal_poloidal", "two_thirds", invs, 32)
