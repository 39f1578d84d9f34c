"""Reference-shaped API over the GB300 library.

Each function keeps the name, arguments, defaults, result type and error behaviour of its
FlowInvariantTransfer.jl counterpart (cited per function); the arithmetic runs in
libfit_gb300 on the GPU. ``spectral`` selects precision through :class:`GB300Spectral`
(``FFTBackend()`` / ``DirectSumBackend()`` are accepted and routed to it); ``execution`` selects
the shell-to-shell form through :class:`GB300Execution`.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .plan import get_plan
from .shells import (coord_is_f32, default_binning, dims_mask, kmax, shell_centers, shell_edges, wavenumber_grid)
from .types import (BandToBandResult, DivergentDecomposition, DirectSumBackend, Enstrophy, FFTBackend, GB300Execution,
                    GB300Spectral, HelicalDecomposition, HelmholtzDecomposition, Helicity, IsotropicShells,
                    KineticEnergy, ModeToModeTransferMethod, ModeToModeTriadResult, NoDecomposition,
                    OrszagTwoThirds, PaddedThreeHalves, PartialFluxResult, PassiveScalar, RotationalDecomposition,
                    ShellToShellResult, ShellToShellTransferMethod, SpectralFluxMethod, SpectralFluxResult,
                    CoarseGrainingFluxMethod,
                    ToroidalPoloidalDecomposition)


def _spec_precision(spectral, arr):
    p = spectral.precision if isinstance(spectral, GB300Spectral) else None
    if p is None:
        p = 32 if np.asarray(arr).dtype == np.complex64 else 64
    if p not in (32, 64):
        raise ValueError("precision must be 32 or 64")
    return p


def _as_component_field(f, nd):
    """``as_component_field`` (``src/Utils.jl:19-26``)."""
    f = np.asarray(f)
    if f.ndim == nd:
        return f[..., None]
    if f.ndim == nd + 1:
        return f
    raise ValueError(f"field has {f.ndim} dims; expected nd={nd} (shape (ns...)) or nd+1={nd + 1} (shape (ns...,1)).")


def _ft(arr):
    return np.float32 if np.asarray(arr).dtype == np.complex64 else np.float64


def _plan(velocity_hat, ks, dealiasing, spectral, advecting_hat):
    if isinstance(spectral, DirectSumBackend) and isinstance(dealiasing, PaddedThreeHalves):
        # the reference's dependency-free backend rejects the exact 3/2 rule (src/NonlinearTerm.jl:106-109)
        raise ValueError("PaddedThreeHalves dealiasing requires the FFT path — pass spectral=FFTBackend() (or "
                         "GB300Spectral()). DirectSumBackend supports only NoDealiasing/OrszagTwoThirds.")
    nd = len(ks)
    v = np.asarray(velocity_hat)
    ns = v.shape[:nd]
    M = v.shape[nd]
    adv = v if advecting_hat is None else np.asarray(advecting_hat)
    D = adv.shape[nd]
    io64 = not (v.dtype == np.complex64 and adv.dtype == np.complex64)
    prec = _spec_precision(spectral, v)
    return get_plan(ns, M, D, dealiasing.key, prec, io64, ks)


def _physical_stack(velocity_fields):
    """(ns..., M) real array from a tuple of M component arrays on one grid, or from one array (a
    single field, M = 1)."""
    if isinstance(velocity_fields, (tuple, list)):
        fields = [np.asarray(f) for f in velocity_fields]
        if not fields:
            raise ValueError("no fields given")
        ns = fields[0].shape
        if any(f.shape != ns for f in fields):
            raise ValueError("velocity components must share one grid shape")
        u = np.stack(fields, axis=-1)
    else:
        u = np.asarray(velocity_fields)[..., None]
    if np.iscomplexobj(u):
        raise ValueError("physical fields must be real")
    if not 1 <= u.ndim - 1 <= 3:
        raise ValueError(f"fields of {u.ndim - 1} dimensions; expected 1, 2 or 3")
    return u


def physical_to_spectral(velocity_fields, spectral=GB300Spectral()):
    """``û = fft(u) ./ Np`` of real physical fields, on the device: the step a caller of the reference
    performs before every spectral diagnostic (``src/FlowInvariantTransfer.jl:233-243``,
    ``cat(FFTW.fft(u), FFTW.fft(v); dims=3) ./ N^2``). ``velocity_fields`` is a tuple of real
    component arrays on one grid, or one real array (a single field). Returns the complex array
    ``(ns..., M)``: complex128 for FP64 (the default for float64 input), complex64 for FP32."""
    u = _physical_stack(velocity_fields)
    ns, M = u.shape[:-1], u.shape[-1]
    prec = spectral.precision if isinstance(spectral, GB300Spectral) and spectral.precision else \
        (32 if u.dtype == np.float32 else 64)
    if prec not in (32, 64):
        raise ValueError("precision must be 32 or 64")
    nd = len(ns)
    ks = wavenumber_grid(ns, (2 * np.pi,) * nd)   # the transform does not depend on the lengths
    # plans carry 1..3 transformed fields (and at least nd advecting ones, unused here): chunks of 3
    parts = []
    for c0 in range(0, M, 3):
        m = min(3, M - c0)
        plan = get_plan(ns, m, max(m, nd), "none", prec, prec == 64, ks)
        parts.append(plan.forward_spectrum(u[..., c0:c0 + m]))
    return parts[0] if len(parts) == 1 else np.concatenate(parts, axis=-1)


def _shells(ks, binning, geometry):
    binning = default_binning(ks) if binning is None else binning
    km = kmax(ks, geometry)
    edges = shell_edges(binning, km)
    centers = shell_centers(binning, km)
    return binning, np.asarray(edges, dtype=np.float64), centers, dims_mask(geometry, len(ks)), coord_is_f32(ks)


# ---- nonlinear term ------------------------------------------------------------------------------
def compute_nonlinear_term(advected_hat, ks, dealiasing=OrszagTwoThirds(), spectral=GB300Spectral(),
                           advecting_hat=None):
    """``compute_nonlinear_term`` (``src/NonlinearTerm.jl:65-76``): N̂ = FFT[(u_adv . grad) f]."""
    f = np.asarray(advected_hat)
    p = _plan(f, ks, dealiasing, spectral, advecting_hat)
    out = p.nonlinear_term(f, advecting_hat)
    return out.astype(f.dtype, copy=False)


def transfer_density(invariant, velocity_hat, N_hat, ks):
    """``transfer_density`` (``src/Invariants.jl:111-118``)."""
    v = np.asarray(velocity_hat)
    p = _plan(v, ks, OrszagTwoThirds(), GB300Spectral(), None)
    return p.transfer_density(invariant.code, v, N_hat).astype(_ft(v))


# ---- decompositions ------------------------------------------------------------------------------
def decompose_field(decomposition, velocity_hat, ks):
    """``decompose_field`` on spectral data (``src/Decomposition.jl:38-141``)."""
    v = np.asarray(velocity_hat)
    if isinstance(decomposition, NoDecomposition):
        return v
    p = _plan(v, ks, OrszagTwoThirds(), GB300Spectral(), None)
    if isinstance(decomposition, HelicalDecomposition):
        up, um = p.helical(v)
        return {"positive": up.astype(v.dtype), "negative": um.astype(v.dtype)}
    if isinstance(decomposition, ToroidalPoloidalDecomposition):
        t, q = p.toroidal_poloidal(v)
        return {"toroidal": t.astype(v.dtype), "poloidal": q.astype(v.dtype)}
    if isinstance(decomposition, (HelmholtzDecomposition, RotationalDecomposition, DivergentDecomposition)):
        r, d = p.helmholtz(v)
        if isinstance(decomposition, RotationalDecomposition):
            return r.astype(v.dtype)
        if isinstance(decomposition, DivergentDecomposition):
            return d.astype(v.dtype)
        return {"rotational": r.astype(v.dtype), "divergent": d.astype(v.dtype)}
    raise ValueError(f"unsupported decomposition {decomposition!r}")


# ---- shells ---------------------------------------------------------------------------------------
def assign_shells_device(ks, binning, geometry=IsotropicShells()):
    """Shell index per mode (Int64, 1-based, 0 = none), computed on the GPU (``src/ShellBinning.jl:126-140``)."""
    binning, edges, _, dm, f32 = _shells(ks, binning, geometry)
    ns = tuple(len(k) for k in ks)
    p = get_plan(ns, 1, len(ks), "none", 64, True, ks)
    return p.assign_shells(edges, dm, f32)


# ---- spectral flux --------------------------------------------------------------------------------
def calculate_spectral_flux(velocity_hat, ks, binning=None, dealiasing=OrszagTwoThirds(), invariant=KineticEnergy(),
                            decomposition=NoDecomposition(), spectral=GB300Spectral(), advecting_hat=None,
                            geometry=IsotropicShells()):
    """``calculate_spectral_flux`` (``src/SpectralFlux.jl:49-122``): T(k_n) and Π = +cumsum(T)."""
    v = np.asarray(velocity_hat)
    binning, edges, centers, dm, f32 = _shells(ks, binning, geometry)
    ft = _ft(v)
    p = _plan(v, ks, dealiasing, spectral, advecting_hat)
    inv = invariant.code
    if isinstance(decomposition, NoDecomposition):
        T, P = p.spectral_flux(v, edges, dm, f32, inv, advecting_hat)
        return SpectralFluxResult(centers.astype(ft), T.astype(ft), np.cumsum(T.astype(ft)).astype(ft))
    dec = decompose_field(decomposition, v, ks)
    if isinstance(dec, dict):
        out = {}
        for name, comp in dec.items():
            T, _ = p.spectral_flux(v, edges, dm, f32, inv, advecting_hat, carrier=comp)
            out[name] = SpectralFluxResult(centers.astype(ft), T.astype(ft), np.cumsum(T.astype(ft)).astype(ft))
        return out
    T, _ = p.spectral_flux(v, edges, dm, f32, inv, advecting_hat, carrier=dec)
    return SpectralFluxResult(centers.astype(ft), T.astype(ft), np.cumsum(T.astype(ft)).astype(ft))


def calculate_scalar_flux(velocity_hat, scalar_hat, ks, binning=None, dealiasing=OrszagTwoThirds(),
                          spectral=GB300Spectral(), geometry=IsotropicShells()):
    """``calculate_scalar_flux`` (``src/SpectralFlux.jl:203-215``)."""
    th = _as_component_field(scalar_hat, len(ks))
    return calculate_spectral_flux(th, ks, binning=binning, dealiasing=dealiasing, invariant=PassiveScalar(),
                                   advecting_hat=velocity_hat, spectral=spectral, geometry=geometry)


# ---- shell-to-shell --------------------------------------------------------------------------------
def calculate_shell_to_shell_transfer(velocity_hat, ks, binning=None, dealiasing=OrszagTwoThirds(),
                                      verify_antisymmetry=True, invariant=KineticEnergy(), spectral=GB300Spectral(),
                                      execution=GB300Execution(), advecting_hat=None, geometry=IsotropicShells()):
    """``calculate_shell_to_shell_transfer`` (``src/ShellToShell/ShellToShellTransfer.jl:78-104``)."""
    v = np.asarray(velocity_hat)
    binning, edges, centers, dm, f32 = _shells(ks, binning, geometry)
    ft = _ft(v)
    p = _plan(v, ks, dealiasing, spectral, advecting_hat)
    mode = _lib.S2S_PLAIN if isinstance(execution, GB300Execution) and execution.mode == "plain" else _lib.S2S_BATCHED
    T, net, asym = p.shell_to_shell(v, edges, dm, f32, invariant.code, mode, verify_antisymmetry, advecting_hat)
    return ShellToShellResult(centers.astype(ft), edges.astype(ft), T.astype(ft), net.astype(ft), ft(asym))


def calculate_scalar_shell_to_shell_transfer(velocity_hat, scalar_hat, ks, **kw):
    """``calculate_scalar_shell_to_shell_transfer`` (``src/ShellToShell/ShellToShellTransfer.jl:143-147``)."""
    th = _as_component_field(scalar_hat, len(ks))
    return calculate_shell_to_shell_transfer(th, ks, invariant=PassiveScalar(), advecting_hat=velocity_hat, **kw)


# ---- smooth band-to-band ----------------------------------------------------------------------------
def calculate_band_to_band_transfer(velocity_hat, ks, bands, dealiasing=OrszagTwoThirds(), invariant=KineticEnergy(),
                                    spectral=GB300Spectral(), advecting_hat=None, geometry=IsotropicShells()):
    """``calculate_band_to_band_transfer`` (``src/BandTransfer.jl:71-113``): smooth T(n,m) between
    the log-Gaussian ``SmoothBands``; returns centers, transfer_matrix, net_transfer,
    max_antisymmetry_error."""
    v = np.asarray(velocity_hat)
    ft = _ft(v)
    p = _plan(v, ks, dealiasing, spectral, advecting_hat)
    T, net, asym = p.band_to_band(v, bands.centers, bands.logwidth, dims_mask(geometry, len(ks)), coord_is_f32(ks),
                                  invariant.code, advecting_hat)
    return BandToBandResult(np.asarray(bands.centers, dtype=ft), T.astype(ft), net.astype(ft), ft(asym))


# ---- partial fluxes --------------------------------------------------------------------------------
def _decomposition_code(decomposition):
    if isinstance(decomposition, HelicalDecomposition):
        return 1, HelicalDecomposition.names
    if isinstance(decomposition, HelmholtzDecomposition):
        return 2, HelmholtzDecomposition.names
    if isinstance(decomposition, ToroidalPoloidalDecomposition):
        return 3, ToroidalPoloidalDecomposition.names
    raise ValueError("calculate_partial_fluxes needs a decomposition that splits u into ≥2 named components "
                     f"(e.g. HelicalDecomposition or HelmholtzDecomposition); got {type(decomposition).__name__}.")


def _partial_result(Tc, names, centers, ft):
    chans = {}
    for sk in range(2):
        for sp in range(2):
            for sq in range(2):
                T = Tc[sk * 4 + sp * 2 + sq].astype(ft)
                chans[(names[sk], names[sp], names[sq])] = SpectralFluxResult(centers.astype(ft), T, np.cumsum(T))
    tot_T = sum(c.transfer_spectrum for c in chans.values())
    tot_P = sum(c.flux for c in chans.values())
    return PartialFluxResult(chans, SpectralFluxResult(centers.astype(ft), tot_T, tot_P), centers.astype(ft))


def calculate_partial_fluxes(velocity_hat, ks, decomposition=HelicalDecomposition(), binning=None,
                             dealiasing=OrszagTwoThirds(), spectral=GB300Spectral(), geometry=IsotropicShells(),
                             invariant=KineticEnergy(), execution=None):
    """``calculate_partial_fluxes`` (``src/SpectralFlux.jl:240-285``): 8 channels (sk, sp, sq) plus the
    total. ``invariant=Helicity()`` swaps the density of ``:277`` (helical helicity channels).
    ``execution=GB300Execution("batched")`` uses the one-pass, graph-replayed form."""
    if isinstance(execution, GB300Execution) and execution.mode == "batched":
        return calculate_partial_fluxes_multi(velocity_hat, ks, invariants=(invariant,), decomposition=decomposition,
                                              binning=binning, dealiasing=dealiasing, spectral=spectral,
                                              geometry=geometry)[type(invariant).__name__]
    v = np.asarray(velocity_hat)
    code, names = _decomposition_code(decomposition)
    binning, edges, centers, dm, f32 = _shells(ks, binning, geometry)
    ft = _ft(v)
    p = _plan(v, ks, dealiasing, spectral, None)
    Tc = p.partial_fluxes(v, code, invariant.code, edges, dm, f32)
    chans = {}
    for sk in range(2):
        for sp in range(2):
            for sq in range(2):
                T = Tc[sk * 4 + sp * 2 + sq].astype(ft)
                chans[(names[sk], names[sp], names[sq])] = SpectralFluxResult(centers.astype(ft), T, np.cumsum(T))
    tot_T = sum(c.transfer_spectrum for c in chans.values())
    tot_P = sum(c.flux for c in chans.values())
    return PartialFluxResult(chans, SpectralFluxResult(centers.astype(ft), tot_T, tot_P), centers.astype(ft))


def calculate_partial_fluxes_multi(velocity_hat, ks, invariants=(KineticEnergy(), Helicity()),
                                   decomposition=HelicalDecomposition(), binning=None, dealiasing=OrszagTwoThirds(),
                                   spectral=GB300Spectral(), geometry=IsotropicShells()):
    """The 8 channels of every invariant in ``invariants`` from one pass over the components (the four
    nonlinear terms are shared), replayed as one CUDA graph from the second call on. Returns
    ``{invariant type name: PartialFluxResult}``, each as ``calculate_partial_fluxes`` would."""
    v = np.asarray(velocity_hat)
    code, names = _decomposition_code(decomposition)
    binning, edges, centers, dm, f32 = _shells(ks, binning, geometry)
    ft = _ft(v)
    p = _plan(v, ks, dealiasing, spectral, None)
    Tc = p.partial_fluxes_batched(v, code, [i.code for i in invariants], edges, dm, f32)
    return {type(inv).__name__: _partial_result(Tc[j], names, centers, ft) for j, inv in enumerate(invariants)}


def calculate_helical_partial_fluxes(velocity_hat, ks, **kw):
    """``calculate_helical_partial_fluxes`` (``src/SpectralFlux.jl:295-296``)."""
    return calculate_partial_fluxes(velocity_hat, ks, decomposition=HelicalDecomposition(), **kw)


# ---- mode-to-mode ------------------------------------------------------------------------------------
def calculate_mode_to_mode_transfer(velocity_hat, ks, invariant=KineticEnergy(), dealiasing=OrszagTwoThirds(),
                                    spectral=GB300Spectral(), max_modes=1024, force=False, advecting_hat=None,
                                    fp64_products=True):
    """``calculate_mode_to_mode_transfer`` (``src/ScaleToScale/ScaleToScaleTransfer.jl:49-91``)."""
    v = np.asarray(velocity_hat)
    nd = len(ks)
    ns = v.shape[:nd]
    nm = int(np.prod(ns))
    if not (force or nm <= max_modes):
        raise ValueError(
            f"calculate_mode_to_mode_transfer resolves S(k|p) over all {nm}×{nm} mode pairs (O(N^{{2D}}) "
            f"time/memory); N_modes={nm} exceeds max_modes={max_modes}. Use calculate_shell_to_shell_transfer / "
            "calculate_spectral_flux for the aggregates, or pass force=true.")
    if isinstance(dealiasing, PaddedThreeHalves):
        raise ValueError("mode-to-mode triads support NoDealiasing and OrszagTwoThirds")
    p = _plan(v, ks, dealiasing, spectral, advecting_hat)
    S, net = p.mode_to_mode(v, invariant.code, fp64_products, advecting_hat)
    ft = _ft(v)
    return ModeToModeTriadResult(invariant, ks, net.astype(ft), S.astype(ft, copy=False))


def calculate_scalar_mode_to_mode_transfer(velocity_hat, scalar_hat, ks, **kw):
    """``calculate_scalar_mode_to_mode_transfer`` (``src/ScaleToScale/ScaleToScaleTransfer.jl:101-105``)."""
    th = _as_component_field(scalar_hat, len(ks))
    return calculate_mode_to_mode_transfer(th, ks, invariant=PassiveScalar(), advecting_hat=velocity_hat, **kw)


# ---- unified dispatch ----------------------------------------------------------------------------
def calculate_energy_transfer(method, velocity_data, coords_or_ks, **kw):
    """``calculate_energy_transfer`` (``src/FlowInvariantTransfer.jl:248-293``): spectral flux,
    shell-to-shell and mode-to-mode take a spectral field and ``ks``; coarse-graining takes a tuple
    of real fields and a tuple of coordinate vectors."""
    if isinstance(method, SpectralFluxMethod):
        return calculate_spectral_flux(velocity_data, coords_or_ks, binning=method.binning, **kw)
    if isinstance(method, ShellToShellTransferMethod):
        return calculate_shell_to_shell_transfer(velocity_data, coords_or_ks, binning=method.binning, **kw)
    if isinstance(method, ModeToModeTransferMethod):
        if method.invariant is not None:
            kw.setdefault("invariant", method.invariant)
        return calculate_mode_to_mode_transfer(velocity_data, coords_or_ks, **kw)
    if isinstance(method, CoarseGrainingFluxMethod):
        from .closure import calculate_coarse_graining_flux
        return calculate_coarse_graining_flux(velocity_data, coords_or_ks, method.scale, method.filter, **kw)
    raise ValueError(f"unsupported method {method!r}")
