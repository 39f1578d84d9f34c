"""GPU parity: every entry point of libfit_gb300 against the CPU oracle on seeded inputs.

Tolerances: FP64 plans agree with the FP64 oracle to 1e-12 relative (max-norm over the output);
FP32 plans (FP32 transforms/products, FP64 reductions) to 1e-5 relative; integer outputs
(shell indices) bit for bit.
"""
import numpy as np
import pytest

import fit_gb300 as F
import oracle as O
from oracle.direct import nonlinear_term_direct

from fields import (curl_noise_3d, e_config1, e_config2, kgrid, scalar_2d, solenoidal_2d, spectrum_field)

pytestmark = pytest.mark.gpu

DEAL = {"none": F.NoDealiasing(), "two_thirds": F.OrszagTwoThirds(), "three_halves": F.PaddedThreeHalves()}
TOL = {64: 1e-12, 32: 1e-5}


def rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("deal", ["none", "two_thirds", "three_halves"])
@pytest.mark.parametrize("N", [8, 12, 16, 24, 64, 96])
def test_nonlinear_term_2d(N, deal, prec):
    u, ks = solenoidal_2d(N, N)
    got = F.compute_nonlinear_term(u, ks, dealiasing=DEAL[deal], spectral=F.GB300Spectral(prec))
    ref = O.nonlinear_term(u, ks, deal)
    assert rel(got, ref) < TOL[prec] * 10


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("deal", ["none", "two_thirds", "three_halves"])
@pytest.mark.parametrize("N", [6, 8, 16, 20])
def test_nonlinear_term_3d_non_hermitian(N, deal, prec):
    u, ks = curl_noise_3d(N, 100 + N)      # complex-noise curl: NOT Hermitian (runtests.jl:509-515)
    got = F.compute_nonlinear_term(u, ks, dealiasing=DEAL[deal], spectral=F.GB300Spectral(prec))
    ref = O.nonlinear_term(u, ks, deal)
    assert rel(got, ref) < TOL[prec] * 10


def test_nonlinear_term_1d_and_direct_sum():
    N = 8
    x = np.arange(N) * 2 * np.pi / N
    uh = (np.fft.fft(np.cos(x) + 0.3 * np.sin(2 * x)) / N)[:, None]
    ks = F.wavenumber_grid((N,), (2 * np.pi,))
    got = F.compute_nonlinear_term(uh, ks, dealiasing=F.NoDealiasing(), spectral=F.GB300Spectral(64))
    assert np.allclose(got, nonlinear_term_direct(uh, ks, truncate=False), atol=1e-12)


@pytest.mark.parametrize("prec", [64, 32])
def test_scalar_advection(prec):
    u, ks = solenoidal_2d(12, 31)
    th = scalar_2d(12, 32)
    got = F.compute_nonlinear_term(th, ks, spectral=F.GB300Spectral(prec), advecting_hat=u)
    assert rel(got, O.nonlinear_term(th, ks, "two_thirds", u)) < TOL[prec] * 10


@pytest.mark.parametrize("ns,dims", [((64, 64), None), ((16, 16, 16), None), ((16, 16, 16), (1, 2)),
                                     ((16, 16, 16), (3,)), ((12, 10), None)])
def test_assign_shells_bit_identical(ns, dims):
    ks = kgrid(ns)
    geo = F.ShellMagnitude(dims)
    for b, ob in [(F.LinearBinning(1.0), ("linear", 1.0)), (F.DyadicBinning(1.0), ("dyadic", 1.0)),
                  (F.LinearBinning(0.7), ("linear", 0.7))]:
        got = F.assign_shells_device(ks, b, geo)
        _, _, _, ref = O.shell_setup(ks, ob, dims)
        assert got.dtype == np.int64 and np.array_equal(got, ref)


def test_spectral_flux_64sq_fp64_config1():
    u, ks = spectrum_field((64, 64), e_config1, seed=1)
    r = F.calculate_spectral_flux(u, ks, binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(64))
    c, T, P = O.spectral_flux(u, ks, ("linear", 1.0), "two_thirds")
    assert len(r.transfer_spectrum) == 46
    assert np.array_equal(r.k_shells, c)
    assert rel(r.transfer_spectrum, T) < 1e-12
    assert np.allclose(r.flux, np.cumsum(r.transfer_spectrum), atol=1e-14)


@pytest.mark.parametrize("inv", ["ke", "enstrophy"])
@pytest.mark.parametrize("deal", ["none", "two_thirds", "three_halves"])
def test_spectral_flux_2d_invariants(inv, deal):
    u, ks = solenoidal_2d(24, 5)
    I = {"ke": F.KineticEnergy(), "enstrophy": F.Enstrophy()}[inv]
    r = F.calculate_spectral_flux(u, ks, binning=F.LinearBinning(1.0), dealiasing=DEAL[deal], invariant=I,
                                  spectral=F.GB300Spectral(64))
    _, T, _ = O.spectral_flux(u, ks, ("linear", 1.0), deal, inv)
    assert rel(r.transfer_spectrum, T) < 1e-11


@pytest.mark.parametrize("inv", ["ke", "helicity", "enstrophy"])
@pytest.mark.parametrize("dims", [None, (1, 2), (3,)])
def test_spectral_flux_3d_non_hermitian(inv, dims):
    u, ks = curl_noise_3d(12, 41)
    I = {"ke": F.KineticEnergy(), "helicity": F.Helicity(), "enstrophy": F.Enstrophy()}[inv]
    r = F.calculate_spectral_flux(u, ks, binning=F.LinearBinning(1.0), invariant=I, spectral=F.GB300Spectral(64),
                                  geometry=F.ShellMagnitude(dims))
    _, T, _ = O.spectral_flux(u, ks, ("linear", 1.0), "two_thirds", inv, dims=dims)
    assert rel(r.transfer_spectrum, T) < 1e-11


@pytest.mark.parametrize("inv", ["ke", "helicity", "enstrophy"])
@pytest.mark.parametrize("deal", ["two_thirds", "three_halves"])
@pytest.mark.parametrize("adv", [False, True])
def test_spectral_flux_live_box_fp32(inv, deal, adv):
    """FP32 cubic plans of a fused transform size compute the flux's nonlinear term on the live box
    (self-advection and a separate advecting field), against the FP64 oracle."""
    F.clear_plans()
    u, ks = curl_noise_3d(64, 43)
    a = curl_noise_3d(64, 44)[0] if adv else None
    I = {"ke": F.KineticEnergy(), "helicity": F.Helicity(), "enstrophy": F.Enstrophy()}[inv]
    r = F.calculate_spectral_flux(u, ks, binning=F.LinearBinning(2.0), invariant=I, dealiasing=DEAL[deal],
                                  spectral=F.GB300Spectral(32), advecting_hat=a)
    _, T, _ = O.spectral_flux(u, ks, ("linear", 2.0), deal, inv, adv_hat=a)
    assert rel(r.transfer_spectrum, T) < 2e-5


def test_scalar_flux_and_decomposed_flux():
    u, ks = solenoidal_2d(16, 32)
    th = scalar_2d(16, 33)
    r = F.calculate_scalar_flux(u, th[..., 0], ks, binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(64))
    _, T, _ = O.spectral_flux(th, ks, ("linear", 1.0), "two_thirds", "scalar", adv_hat=u)
    assert rel(r.transfer_spectrum, T) < 1e-11
    u3, ks3 = curl_noise_3d(12, 51)
    rh = F.calculate_spectral_flux(u3, ks3, binning=F.LinearBinning(1.0), decomposition=F.HelicalDecomposition(),
                                   spectral=F.GB300Spectral(64))
    comps = O.helical_decompose(u3, ks3)
    for name in ("positive", "negative"):
        _, T, _ = O.spectral_flux(u3, ks3, ("linear", 1.0), "two_thirds", carrier=comps[name])
        assert rel(rh[name].transfer_spectrum, T) < 1e-11


@pytest.mark.parametrize("field", ["reference", "solenoidal"])
def test_execution_forms_agree(field):     # runtests.jl:993-1023
    """The reference's serial/threaded/distributed parity check: the plain and batched FP64 forms
    agree to 1e-12 (absolute on its field, u = (cos x, cos y) on 8^2, whose transfer the 2/3 rule
    removes entirely; relative to max|T| on a random solenoidal 16^2 field), as its execution
    backends do, and both equal the oracle; the batched FP32 form is within FP32 rounding.
    LinearBinning(1), 2/3 rule."""
    if field == "reference":
        N = 8
        ks = F.wavenumber_grid((N, N), (2 * np.pi,) * 2)
        u = np.zeros((N, N, 2), complex)
        u[1, 0, 0] = u[N - 1, 0, 0] = 0.5
        u[0, 1, 1] = u[0, N - 1, 1] = 0.5
    else:
        u, ks = solenoidal_2d(16, 17)
    b = F.LinearBinning(1.0)
    r = {(p, m): F.calculate_shell_to_shell_transfer(u, ks, binning=b, spectral=F.GB300Spectral(p),
                                                     execution=F.GB300Execution(m))
         for p, m in ((64, "plain"), (64, "batched"), (32, "batched"))}
    _, _, T, net, _ = O.shell_to_shell(u, ks, ("linear", 1.0), "two_thirds")
    scale = max(np.abs(T).max(), 1.0) if field == "reference" else np.abs(T).max()
    assert field == "reference" or scale > 0
    a, c = r[(64, "plain")], r[(64, "batched")]
    assert np.max(np.abs(a.transfer_matrix - c.transfer_matrix)) <= 1e-12 * scale
    assert np.max(np.abs(a.net_transfer - c.net_transfer)) <= 1e-12 * scale
    assert np.max(np.abs(a.transfer_matrix - T)) <= 1e-12 * scale
    assert np.max(np.abs(a.net_transfer - net)) <= 1e-12 * scale
    assert np.max(np.abs(r[(32, "batched")].transfer_matrix - T)) <= 1e-5 * scale


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("mode", ["plain", "batched"])
@pytest.mark.parametrize("deal", ["none", "two_thirds", "three_halves"])
def test_shell_to_shell_2d(prec, mode, deal):
    u, ks = solenoidal_2d(16, 13)
    r = F.calculate_shell_to_shell_transfer(u, ks, binning=F.LinearBinning(1.0), dealiasing=DEAL[deal],
                                            spectral=F.GB300Spectral(prec), execution=F.GB300Execution(mode))
    _, _, T, net, asym = O.shell_to_shell(u, ks, ("linear", 1.0), deal)
    assert rel(r.transfer_matrix, T) < TOL[prec] * 10
    assert rel(r.net_transfer, net) < TOL[prec] * 100


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("deal", ["two_thirds", "three_halves"])
@pytest.mark.parametrize("inv", ["ke", "helicity"])
def test_shell_to_shell_3d(prec, deal, inv):
    u, ks = spectrum_field((16, 16, 16), e_config2, seed=3)
    I = {"ke": F.KineticEnergy(), "helicity": F.Helicity()}[inv]
    for mode in ("plain", "batched", "batched", "batched"):   # eager, capture, replay, replay
        r = F.calculate_shell_to_shell_transfer(u, ks, binning=F.LinearBinning(2.0), dealiasing=DEAL[deal],
                                                invariant=I, spectral=F.GB300Spectral(prec),
                                                execution=F.GB300Execution(mode))
        _, _, T, _, _ = O.shell_to_shell(u, ks, ("linear", 2.0), deal, inv)
        assert rel(r.transfer_matrix, T) < TOL[prec] * 10, mode


def test_scalar_shell_to_shell():
    u, ks = solenoidal_2d(16, 14)
    th = scalar_2d(16, 15)
    r = F.calculate_scalar_shell_to_shell_transfer(u, th, ks, binning=F.LinearBinning(1.0),
                                                   spectral=F.GB300Spectral(64))
    _, _, T, _, _ = O.shell_to_shell(th, ks, ("linear", 1.0), "two_thirds", "scalar", adv_hat=u)
    assert rel(r.transfer_matrix, T) < 1e-11


@pytest.mark.parametrize("prec", [64, 32])
def test_helical_partial_fluxes(prec):
    u, ks = curl_noise_3d(12, 91)
    for inv, oinv in ((F.KineticEnergy(), "ke"), (F.Helicity(), "helicity")):
        r = F.calculate_partial_fluxes(u, ks, binning=F.LinearBinning(1.0), spectral=F.GB300Spectral(prec),
                                       invariant=inv)
        chans, _, _ = O.partial_fluxes(u, ks, "helical", ("linear", 1.0), "two_thirds", invariant=oinv)
        scale = max(np.max(np.abs(c[0])) for c in chans.values())
        for key, (T, _) in chans.items():
            got = r.channels[key].transfer_spectrum
            assert np.max(np.abs(got - T)) < TOL[prec] * 10 * scale, key


def test_helmholtz_partial_fluxes():
    u, ks = solenoidal_2d(16, 92)
    r = F.calculate_partial_fluxes(u, ks, decomposition=F.HelmholtzDecomposition(), binning=F.LinearBinning(1.0),
                                   spectral=F.GB300Spectral(64))
    chans, _, _ = O.partial_fluxes(u, ks, "helmholtz", ("linear", 1.0), "two_thirds")
    scale = max(np.max(np.abs(c[0])) for c in chans.values())
    for key, (T, _) in chans.items():
        assert np.max(np.abs(r.channels[key].transfer_spectrum - T)) < 1e-11 * scale


@pytest.mark.parametrize("fp64", [True, False])
def test_mode_to_mode(fp64):
    u, ks = solenoidal_2d(12, 21)
    r = F.calculate_mode_to_mode_transfer(u, ks, spectral=F.GB300Spectral(64), fp64_products=fp64)
    net, S = O.mode_to_mode_triad(u, ks, "two_thirds")
    tol = 1e-12 if fp64 else 1e-5
    assert rel(r.transfer, S) < tol * 10
    assert rel(r.net_transfer, net) < tol * 100
    u3, ks3 = curl_noise_3d(6, 7)
    for inv, oi in ((F.KineticEnergy(), "ke"), (F.Helicity(), "helicity")):
        r3 = F.calculate_mode_to_mode_transfer(u3, ks3, invariant=inv, force=True, fp64_products=fp64)
        _, S3 = O.mode_to_mode_triad(u3, ks3, "two_thirds", oi)
        assert rel(r3.transfer, S3) < tol * 10


def test_transfer_density_and_decompositions():
    u, ks = curl_noise_3d(8, 3)
    Nh = O.nonlinear_term(u, ks, "two_thirds")
    for inv, oi in ((F.KineticEnergy(), "ke"), (F.Helicity(), "helicity"), (F.Enstrophy(), "enstrophy")):
        assert rel(F.transfer_density(inv, u, Nh, ks), O.transfer_density(oi, u, Nh, ks)) < 1e-12
    d = F.decompose_field(F.HelicalDecomposition(), u, ks)
    o = O.helical_decompose(u, ks)
    assert rel(d["positive"], o["positive"]) < 1e-12 and rel(d["negative"], o["negative"]) < 1e-12
    u2, ks2 = solenoidal_2d(8, 4)
    h = F.decompose_field(F.HelmholtzDecomposition(), u2, ks2)
    oh = O.helmholtz_decompose(u2, ks2)
    assert rel(h["rotational"], oh["rotational"]) < 1e-12


def test_errors_match_reference_behaviour():
    u, ks = solenoidal_2d(8, 1)
    with pytest.raises(ValueError):
        F.calculate_spectral_flux(u, ks, invariant=F.Helicity())      # Helicity is 3D only
    with pytest.raises(ValueError):
        F.calculate_mode_to_mode_transfer(np.zeros((64, 64, 2), complex), kgrid((64, 64)))  # > max_modes
    with pytest.raises(ValueError):
        F.calculate_spectral_flux(u, ks, geometry=F.ParallelShells())   # dims=(3,) in 2D


def test_zero_field_gives_zero():
    ks = kgrid((6, 6))
    r = F.calculate_shell_to_shell_transfer(np.zeros((6, 6, 2), complex), ks, binning=F.LinearBinning(1.0),
                                            dealiasing=F.NoDealiasing(), verify_antisymmetry=False)
    assert np.all(np.abs(r.transfer_matrix) < 1e-14) and np.isnan(r.max_antisymmetry_error)


@pytest.mark.parametrize("deal", ["two_thirds", "three_halves"])
@pytest.mark.parametrize("inv", ["ke", "helicity"])
@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("xpass", ["register", "staged"])
def test_fused_shell_to_shell_64(deal, inv, herm, xpass, monkeypatch):
    """The fused FP32 pipeline (cubic grid of a compiled size) against the FP64 oracle, with both
    forms of its x pass (register-accumulating and shared-memory staged)."""
    if xpass == "staged":
        monkeypatch.setenv("FIT_XMIX_BULK", "1")
    F.clear_plans()
    if herm:
        u, ks = spectrum_field((64, 64, 64), e_config2, seed=5)
    else:
        u, ks = curl_noise_3d(64, 6)
    I = {"ke": F.KineticEnergy(), "helicity": F.Helicity()}[inv]
    r = F.calculate_shell_to_shell_transfer(u, ks, binning=F.LinearBinning(4.0), dealiasing=DEAL[deal], invariant=I,
                                            spectral=F.GB300Spectral(32), execution=F.GB300Execution("batched"))
    _, _, T, net, _ = O.shell_to_shell(u, ks, ("linear", 4.0), deal, inv)
    assert rel(r.transfer_matrix, T) < 1e-5
    assert rel(r.net_transfer, net) < 1e-4


@pytest.mark.parametrize("n", [96, 128])
@pytest.mark.parametrize("inv", ["ke", "helicity"])
def test_fused_shell_to_shell_even_kx(n, inv):
    """The fused pipeline on grids whose live box has an even number of x frequencies (96: KX = 32,
    128: KX = 42; the x pass then pairs lines (c, c + C)) against the FP64 oracle."""
    F.clear_plans()
    u, ks = spectrum_field((n, n, n), e_config2, seed=11)
    I = {"ke": F.KineticEnergy(), "helicity": F.Helicity()}[inv]
    dk = n / 12.0
    r = F.calculate_shell_to_shell_transfer(u, ks, binning=F.LinearBinning(dk), invariant=I,
                                            spectral=F.GB300Spectral(32), execution=F.GB300Execution("batched"))
    _, _, T, net, _ = O.shell_to_shell(u, ks, ("linear", dk), "two_thirds", inv)
    assert rel(r.transfer_matrix, T) < 1e-5
    assert rel(r.net_transfer, net) < 1e-4


def test_fused_host_input_reads_only_kept_modes():
    """The fused 2/3 path copies only the kept slabs of a host field: values outside the kept box
    (NaN here) must not reach the result, which equals the clean field's and the oracle's."""
    F.clear_plans()
    u, ks = spectrum_field((64, 64, 64), e_config2, seed=7)
    kw = dict(binning=F.LinearBinning(4.0), dealiasing=F.OrszagTwoThirds(), spectral=F.GB300Spectral(32),
              execution=F.GB300Execution("batched"))
    clean = F.calculate_shell_to_shell_transfer(u, ks, **kw).transfer_matrix
    idx = np.arange(64)
    kept = np.minimum(idx, 64 - idx) < 64 // 3
    box = kept[:, None, None] & kept[None, :, None] & kept[None, None, :]
    dirty = u.copy()
    dirty[~box] = np.nan
    got = F.calculate_shell_to_shell_transfer(dirty, ks, **kw).transfer_matrix
    assert np.all(np.isfinite(got))
    assert np.array_equal(got, clean)
    _, _, T, _, _ = O.shell_to_shell(u, ks, ("linear", 4.0), "two_thirds")
    assert rel(got, T) < 1e-5


@pytest.mark.parametrize("n,deal", [(512, "two_thirds"), (256, "three_halves"), (128, "three_halves"),
                                    (512, "three_halves")])
def test_fused_shell_to_shell_largest_tiles(n, deal):
    """The fused pipeline at the transform lengths with their own tiles (512: 2/3 rule at 512^3; 384:
    the 3/2 rule at 256^3) and at the other 3/2 lengths (192 at 128^3, 768 at 512^3: two mediators
    per batch) against the plan's FP64 path on the same device field (device pointers, a few wide
    shells so that the FP64 path stays short)."""
    torch = pytest.importorskip("torch")
    F.clear_plans()
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    ns = (n, n, n)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = torch.randn((3, n, n, n), device=dev, dtype=torch.complex64, generator=g)
    edges = np.asarray(F.shell_edges(F.LinearBinning(n / 8.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    out = {}
    for prec, mode, field in ((32, F._lib.S2S_BATCHED, u), (64, F._lib.S2S_PLAIN, u.to(torch.complex128))):
        plan = F.Plan(ns, 3, 3, deal, prec, prec == 64, ks)
        T = torch.zeros((nsh, nsh), dtype=torch.float64, device=dev)
        plan.shell_to_shell_device(field.data_ptr(), 0, edges, 7, 0, 0, mode, T.data_ptr(), 0, 0)
        torch.cuda.synchronize()
        out[prec] = T.cpu().numpy()
        del plan, T
        F.clear_plans()
    assert np.max(np.abs(out[64])) > 0
    assert rel(out[32], out[64]) < 1e-5


@pytest.mark.parametrize("inv", ["ke", "helicity"])
def test_fused_shell_to_shell_two_batches(inv):
    """28 shells at 64^3: more mediators than one batch holds (16), so the sequence runs two batches;
    the first (eager), second (captured) and third (replayed) calls all equal the FP64 oracle."""
    F.clear_plans()
    u, ks = spectrum_field((64, 64, 64), e_config2, seed=9)
    I = {"ke": F.KineticEnergy(), "helicity": F.Helicity()}[inv]
    _, _, T, net, _ = O.shell_to_shell(u, ks, ("linear", 2.0), "two_thirds", inv)
    assert T.shape[0] > 16
    for _ in range(3):
        r = F.calculate_shell_to_shell_transfer(u, ks, binning=F.LinearBinning(2.0), invariant=I,
                                                spectral=F.GB300Spectral(32), execution=F.GB300Execution("batched"))
        assert rel(r.transfer_matrix, T) < 1e-5
        assert rel(r.net_transfer, net) < 1e-4


@pytest.mark.parametrize("seed", [3, 11])
def test_fused_shell_to_shell_conservation_floor(seed):
    """Energy conservation of the raw FP32 pipeline on an exactly solenoidal FP64 input (FP64 host
    buffers, FP32 arithmetic): sum_nm T(n,m) vanishes in exact arithmetic for a divergence-free,
    dealiased field, so |sum T| / sum |T| measures the pipeline's own rounding. The FP32 figure
    stays at the single-precision floor (measured 3.1e-8 and 3.6e-8 on GB300 for these two fields) and
    the FP64 path on the same field at the double-precision floor (below 1e-16)."""
    F.clear_plans()
    u, ks = spectrum_field((64, 64, 64), e_config2, seed=seed)
    assert u.dtype == np.complex128
    b = F.LinearBinning(2.0)
    res = {}
    for prec, ex in ((32, "batched"), (64, "plain")):
        r = F.calculate_shell_to_shell_transfer(u, ks, binning=b, spectral=F.GB300Spectral(prec),
                                                execution=F.GB300Execution(ex))
        T = np.asarray(r.transfer_matrix, dtype=np.float64)
        res[prec] = (T, abs(T.sum()) / np.abs(T).sum())
    print(f"seed {seed}: conservation FP32 {res[32][1]:.3e}, FP64 {res[64][1]:.3e}, "
          f"FP32 vs FP64 {rel(res[32][0], res[64][0]):.3e}")
    assert res[64][1] < 1e-12
    assert res[32][1] < 3e-7
    assert rel(res[32][0], res[64][0]) < 1e-5


def test_fused_shell_to_shell_shells_without_kept_modes():
    """Shells that hold no mode of the 2/3-kept box (64^3: kept |k_d| <= 20, so |k| <= 34.7) leave no
    mediator for the fused batched form, and every T(n, m) is a sum over no triad: eager, captured
    and replayed calls, from a host array and from a pinned host buffer, return all zeros."""
    torch = pytest.importorskip("torch")
    F.clear_plans()
    n = 64
    u, ks = spectrum_field((n, n, n), e_config2, seed=4)
    edges = np.array([40.0, 45.0, 50.0])
    plan = F.Plan((n, n, n), 3, 3, "two_thirds", 32, False, ks)
    pinned = torch.empty((3, n, n, n), dtype=torch.complex64, pin_memory=True)
    host = np.transpose(pinned.numpy(), (3, 2, 1, 0))
    host[...] = u.astype(np.complex64)
    for arr in (np.asfortranarray(u.astype(np.complex64)), host):
        for _ in range(3):
            T, net, _ = plan.shell_to_shell(arr, edges, 7, 0, 0, F._lib.S2S_BATCHED)
            assert T.shape == (2, 2) and not np.any(T) and not np.any(net)
