"""Golden fixtures (tests/golden/golden.npz, written by tests/golden/make_golden.py from the oracle).

CPU: the oracle still reproduces its committed outputs. GPU: the CUDA path matches the fixtures
(FP64 plans to 1e-12 relative, FP32 plans to 1e-5, shell indices bit for bit)."""
import os

import numpy as np
import pytest

import fit_gb300 as F
import oracle as O
from fields import kgrid

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz"))


def rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300)


def test_oracle_reproduces_fixtures():
    ks = kgrid((64, 64))
    c, T, P = O.spectral_flux(G["flux64_u"], ks, ("linear", 1.0), "two_thirds")
    assert rel(T, G["flux64_T"]) < 1e-13 and np.array_equal(c, G["flux64_centers"])
    ks3 = kgrid((12, 12, 12))
    assert rel(O.nonlinear_term(G["nl12_u"], ks3, "three_halves"), G["nl12_three_halves_N"]) < 1e-13
    ks16 = kgrid((16, 16, 16))
    _, _, T16, _, _ = O.shell_to_shell(G["s2s16_u"], ks16, ("linear", 2.0), "two_thirds")
    assert rel(T16, G["s2s16_two_thirds_T"]) < 1e-13


@pytest.mark.gpu
def test_gpu_flux_and_shells_match_fixture():
    ks = kgrid((64, 64))
    r = F.calculate_spectral_flux(G["flux64_u"], ks, binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(64))
    assert rel(r.transfer_spectrum, G["flux64_T"]) < 1e-12
    assert np.array_equal(F.assign_shells_device(ks, F.LinearBinning(1.0)), G["flux64_sidx"])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [64, 32])
def test_gpu_nonlinear_and_s2s_match_fixture(prec):
    tol = 1e-12 if prec == 64 else 1e-5
    ks3 = kgrid((12, 12, 12))
    for d, D in (("none", F.NoDealiasing()), ("two_thirds", F.OrszagTwoThirds()),
                 ("three_halves", F.PaddedThreeHalves())):
        got = F.compute_nonlinear_term(G["nl12_u"], ks3, dealiasing=D, spectral=F.GB300Spectral(prec))
        assert rel(got, G[f"nl12_{d}_N"]) < tol * 10
    ks16 = kgrid((16, 16, 16))
    for d, D in (("two_thirds", F.OrszagTwoThirds()), ("three_halves", F.PaddedThreeHalves())):
        r = F.calculate_shell_to_shell_transfer(G["s2s16_u"], ks16, binning=F.LinearBinning(2.0), dealiasing=D,
                                                spectral=F.GB300Spectral(prec))
        assert rel(r.transfer_matrix, G[f"s2s16_{d}_T"]) < tol * 10


@pytest.mark.gpu
def test_gpu_partial_fluxes_and_m2m_match_fixture():
    ks3 = kgrid((12, 12, 12))
    r = F.calculate_partial_fluxes(G["nl12_u"], ks3, binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(64))
    got = np.stack([r.channels[(a, b, c)].transfer_spectrum for a in ("positive", "negative")
                    for b in ("positive", "negative") for c in ("positive", "negative")])
    assert np.max(np.abs(got - G["pf12_T"])) < 1e-11 * np.max(np.abs(G["pf12_T"]))
    ks2 = kgrid((12, 12))
    m = F.calculate_mode_to_mode_transfer(G["m2m12_u"], ks2, spectral=F.GB300Spectral(64))
    assert rel(m.transfer, G["m2m12_S"]) < 1e-11 and rel(m.net_transfer, G["m2m12_net"]) < 1e-10
