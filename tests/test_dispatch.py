"""The reference's unified-dispatch, Float32-propagation and mode-to-mode guard testsets
(``test/runtests.jl:695-715``, ``:779-805`` and ``:1056-1069``) through this package:
``calculate_energy_transfer`` routes each method type to its calculation and returns that
calculation's result type; Float32 box lengths give Float32 wavenumbers, shell coordinates, edges
and centres, and a ComplexF32 field gives Float32 results; mode-to-mode rejects helicity in 2D and
accepts enstrophy in 3D and kinetic energy in both."""
import numpy as np
import pytest

import fit_gb300 as F


def test_float32_shell_helpers():          # runtests.jl:779-790
    N = 8
    Ls = (np.float32(2 * np.pi),) * 2
    ks = F.wavenumber_grid((N, N), Ls)
    assert ks[0].dtype == np.float32 and ks[1].dtype == np.float32
    km = F.kmax(ks)
    assert isinstance(km, np.float32)
    b = F.LinearBinning(np.float32(2 * np.pi) / N)
    assert F.shell_edges(b, km).dtype == np.float32
    assert F.shell_centers(b, km).dtype == np.float32


def test_dispatch_rejects_unknown_methods():
    with pytest.raises(ValueError):
        F.calculate_energy_transfer(object(), np.zeros((8, 1), complex), F.wavenumber_grid((8,), (2 * np.pi,)))


@pytest.mark.gpu
def test_unified_dispatch():               # runtests.jl:695-715
    N, L = 8, 2 * np.pi
    ks = F.wavenumber_grid((N,), (L,))
    u = np.zeros((N, 1), complex)
    r1 = F.calculate_energy_transfer(F.SpectralFluxMethod(F.LinearBinning(2 * np.pi / L)), u, ks)
    assert isinstance(r1, F.SpectralFluxResult)
    r2 = F.calculate_energy_transfer(F.ShellToShellTransferMethod(F.LinearBinning(2 * np.pi / L)), u, ks)
    assert isinstance(r2, F.ShellToShellResult)
    x = np.array([L * i / N for i in range(N)])
    r3 = F.calculate_energy_transfer(F.CoarseGrainingFluxMethod(F.GaussianFilter(), np.pi / 2),
                                     (np.zeros((N, N)), np.zeros((N, N))), (x, x))
    assert isinstance(r3, F.CoarseGrainingFluxResult)
    # mode-to-mode through the dispatch carries the method's invariant (helicity is 3D only)
    u3 = np.zeros((4, 4, 4, 3), complex)
    ks3 = F.wavenumber_grid((4, 4, 4), (L, L, L))
    r4 = F.calculate_energy_transfer(F.ModeToModeTransferMethod(invariant=F.KineticEnergy()), u3, ks3)
    direct = F.calculate_mode_to_mode_transfer(u3, ks3, invariant=F.KineticEnergy())
    assert type(r4) is type(direct)
    with pytest.raises(ValueError):
        F.calculate_energy_transfer(F.ModeToModeTransferMethod(invariant=F.Helicity()), np.zeros((4, 4, 2), complex),
                                    F.wavenumber_grid((4, 4), (L, L)))


@pytest.mark.gpu
def test_float32_results():                # runtests.jl:791-804
    N = 8
    Ls = (np.float32(2 * np.pi),) * 2
    ks = F.wavenumber_grid((N, N), Ls)
    b = F.LinearBinning(np.float32(2 * np.pi) / N)
    u = np.zeros((N, N, 2), np.complex64)
    r = F.calculate_spectral_flux(u, ks, binning=b, dealiasing=F.NoDealiasing(), spectral=F.DirectSumBackend())
    assert isinstance(r, F.SpectralFluxResult)
    assert r.k_shells.dtype == np.float32 and r.transfer_spectrum.dtype == np.float32
    th = np.zeros((N, N), np.complex64)
    rt = F.calculate_scalar_flux(u, th, ks, binning=b, dealiasing=F.NoDealiasing(), spectral=F.DirectSumBackend())
    assert rt.transfer_spectrum.dtype == np.float32


@pytest.mark.gpu
def test_mode_to_mode_guards():            # runtests.jl:1056-1069
    L = 2 * np.pi
    ks2 = F.wavenumber_grid((4, 4), (L, L))
    u2 = np.zeros((4, 4, 2), complex)
    u2[1, 0, 0] = 0.5
    u2[0, 1, 1] = 0.5
    with pytest.raises(ValueError):      # Helicity is 3D only
        F.calculate_mode_to_mode_transfer(u2, ks2, invariant=F.Helicity())
    ks3 = F.wavenumber_grid((4, 4, 4), (L, L, L))
    u3 = np.zeros((4, 4, 4, 3), complex)
    u3[1, 0, 0, 0] = 0.5
    assert isinstance(F.calculate_mode_to_mode_transfer(u3, ks3, invariant=F.Enstrophy()), F.ModeToModeTriadResult)
    assert isinstance(F.calculate_mode_to_mode_transfer(u2, ks2, invariant=F.KineticEnergy()), F.ModeToModeTriadResult)
    assert isinstance(F.calculate_mode_to_mode_transfer(u3, ks3, invariant=F.KineticEnergy()), F.ModeToModeTriadResult)
