"""FP64 numpy restatement of FlowInvariantTransfer.jl's transfer hot path (TEST ORACLE ONLY).

Every function cites the reference file:line it restates. Conventions follow the reference:

* arrays are indexed ``[x, y, (z,) component]`` (Julia column-major ``(ns..., comp)``);
* ``û = fft(u)/Np`` (or raw ``fft``: every diagnostic is linear in each factor);
* wavenumbers are in FFTW order with ``+N/2`` at the Nyquist index (``Utils.jl:51-63``).

The transforms are ``numpy.fft`` (pocketfft, FP64), standing in for FFTW Float64: both are
~1e-16-accurate DFTs, so the differences are far below every tolerance used in the tests.

Spec objects are plain tuples so that the oracle depends on nothing in the product package:

* binning: ``("linear", dk)``, ``("log", k0, lam)``, ``("dyadic", k0)``, ``("custom", edges)``
* geometry: ``None`` (isotropic) or a tuple of 1-based dims, e.g. ``(1, 2)``, ``(3,)``
* dealiasing: ``"none"``, ``"two_thirds"``, ``"three_halves"``
* invariant: ``"ke"``, ``"scalar"``, ``"helicity"``, ``"enstrophy"``
"""
from __future__ import annotations

import math

import numpy as np

_WORKERS = None


def set_fft_workers(n):
    """Use scipy.fft with ``n`` threads for every transform (the reference uses FFTW threads /
    OhMyThreads for the same transforms); ``None`` restores single-threaded numpy.fft."""
    global _WORKERS
    _WORKERS = n


def _fftn(a, axes):
    if _WORKERS:
        import scipy.fft as sf
        return sf.fftn(a, axes=axes, workers=_WORKERS)
    return np.fft.fftn(a, axes=axes)


def _ifftn(a, axes):
    if _WORKERS:
        import scipy.fft as sf
        return sf.ifftn(a, axes=axes, workers=_WORKERS)
    return np.fft.ifftn(a, axes=axes)


__all__ = [
    "wavenumber_grid", "keep_mask", "shell_coordinate", "julia_range", "shell_edges",
    "shell_centers", "assign_shells", "padded_len", "embed_spectrum", "truncate_spectrum",
    "nonlinear_term", "dealias_copy", "transfer_density", "spectral_flux", "shell_to_shell",
    "helical_decompose", "toroidal_poloidal_decompose", "helmholtz_decompose", "partial_fluxes",
    "mode_to_mode", "mode_to_mode_triad", "default_binning", "filter_response",
    "coarse_graining_flux", "shell_setup", "set_fft_workers", "s2s_setup", "s2s_column",
    "band_weights", "band_to_band",
]


# ---------------------------------------------------------------------------------------------
# Wavenumbers, masks, shells
# ---------------------------------------------------------------------------------------------

def wavenumber_grid(ns, Ls, dtype=np.float64):
    """FFTW-order wavenumbers, +N/2 at the Nyquist index. Restates ``src/Utils.jl:51-63``."""
    out = []
    for N, L in zip(ns, Ls):
        dk = dtype(2 * np.pi) / dtype(L)
        idx = np.arange(N)
        km = np.where(idx <= N // 2, idx, idx - N).astype(dtype)
        out.append((km * dk).astype(dtype))
    return tuple(out)


def keep_mask(ns):
    """True where a mode survives the 2/3 rule: every |k_d| index < N_d ÷ 3.

    Restates ``_is_dealiased`` (``src/NonlinearTerm.jl:134-141``): integer ``N÷3`` cutoff on the
    FFTW-order index magnitude (the float ``N/3`` of ``Utils.dealiasing_mask`` is NOT used)."""
    keep = np.ones(tuple(ns), dtype=bool)
    for d, N in enumerate(ns):
        idx = np.arange(N)
        kabs = np.where(idx <= N // 2, idx, N - idx)
        shape = [1] * len(ns)
        shape[d] = N
        keep &= (kabs < N // 3).reshape(shape)
    return keep


def _kcomp(ks, d, ns):
    shape = [1] * len(ns)
    shape[d] = ns[d]
    return np.asarray(ks[d]).reshape(shape)


def shell_coordinate(ks, dims=None):
    """sqrt(sum_{d in dims} k_d^2) per mode, accumulated in dims order.

    Restates ``shell_coordinate(::ShellMagnitude, ks)`` (``src/ShellBinning.jl:19-36``),
    including the ArgumentError for a dim outside ``1:nd``."""
    nd = len(ks)
    ns = tuple(len(k) for k in ks)
    dims = tuple(range(1, nd + 1)) if dims is None else tuple(dims)
    if not all(1 <= d <= nd for d in dims):
        raise ValueError(f"ShellMagnitude dims={dims} out of range for nd={nd} spatial dimensions.")
    ft = np.asarray(ks[0]).dtype
    s = np.zeros(ns, dtype=ft)
    for d in dims:
        kd = _kcomp(ks, d - 1, ns).astype(ft)
        s = s + kd * kd
    return np.sqrt(s)


def julia_range(start, step, stop):
    """Elements of Julia's float range ``start:step:stop`` (as ``collect`` returns them).

    The length is the largest ``len`` with ``start + (len-1)*step <= stop`` (Julia's rational
    and fallback constructors agree on it for the ranges built by ``shell_edges``), and every
    element is the correctly rounded ``start + i*step``."""
    start = float(start); step = float(step); stop = float(stop)
    if step == 0:
        raise ValueError("range step cannot be zero")
    lf = (stop - start) / step
    if lf < 0:
        return np.zeros(0)
    n = int(math.floor(lf)) + 1
    while n > 0 and start + (n - 1) * step > stop:
        n -= 1
    while start + n * step <= stop:
        n += 1
    return start + np.arange(n, dtype=np.float64) * step


def shell_edges(binning, kmax):
    """Shell edges. Restates ``src/ShellBinning.jl:50-79`` (Linear :50-57, Log :59-70,
    Dyadic :72-74, Custom :76-79)."""
    kind = binning[0]
    if kind == "linear":
        dk = float(binning[1])
        if not dk > 0:
            raise ValueError("LinearBinning: Δk must be positive.")
        if not kmax > 0:
            raise ValueError("k_max must be positive.")
        edges = list(julia_range(0.0, dk, kmax))
        if edges[-1] < kmax:
            edges.append(float(kmax))
        return np.asarray(edges, dtype=np.float64)
    if kind in ("log", "dyadic"):
        k0 = float(binning[1])
        lam = 2.0 if kind == "dyadic" else float(binning[2])
        if not k0 > 0:
            raise ValueError("LogarithmicBinning: k₀ must be positive.")
        if not lam > 1:
            raise ValueError("LogarithmicBinning: λ must be > 1.")
        if not kmax >= k0:
            raise ValueError("k_max must be >= k₀.")
        n_max = int(math.floor(math.log(kmax / k0) / math.log(lam)))
        edges = [k0 * lam ** n for n in range(0, n_max + 2)]
        while len(edges) > 2 and edges[-2] > kmax:
            edges.pop()
        return np.asarray(edges, dtype=np.float64)
    if kind == "custom":
        e = np.asarray(binning[1], dtype=np.float64)
        if not np.all(np.diff(e) >= 0):
            raise ValueError("CustomBinning: edges must be monotonically increasing.")
        return e
    raise ValueError(f"unknown binning {binning!r}")


def shell_centers(binning, kmax):
    """Geometric mean for log/dyadic, arithmetic otherwise (``src/ShellBinning.jl:91-106``)."""
    e = shell_edges(binning, kmax)
    if len(e) - 1 <= 0:
        raise ValueError(f"No shells within k_max={kmax} for this binning.")
    if binning[0] in ("log", "dyadic"):
        return np.sqrt(e[:-1] * e[1:])
    return (e[:-1] + e[1:]) / 2


def assign_shells(kmag, edges):
    """1-based shell index, 0 when outside every shell; first match wins.
    Restates ``assign_shells`` (``src/ShellBinning.jl:126-140``)."""
    idx = np.zeros(kmag.shape, dtype=np.int64)
    done = np.zeros(kmag.shape, dtype=bool)
    for n in range(len(edges) - 1):
        hit = (~done) & (edges[n] <= kmag) & (kmag < edges[n + 1])
        idx[hit] = n + 1
        done |= hit
    return idx


def default_binning(ks):
    """``LinearBinning(min |k| > 0)`` (``src/SpectralFlux.jl:301-313``)."""
    m = math.inf
    for k in ks:
        a = np.abs(np.asarray(k, dtype=np.float64))
        a = a[a > 0]
        if a.size:
            m = min(m, float(a.min()))
    return ("linear", m if math.isfinite(m) else 1.0)


def shell_setup(ks, binning, dims=None):
    """(coordinate, edges, centers, shell index) exactly as every diagnostic builds them
    (e.g. ``src/SpectralFlux.jl:105-108``)."""
    kc = shell_coordinate(ks, dims)
    kmax = float(kc.max())
    edges = shell_edges(binning, kmax)
    centers = shell_centers(binning, kmax)
    return kc, edges, centers, assign_shells(kc, edges)


# ---------------------------------------------------------------------------------------------
# Nonlinear term
# ---------------------------------------------------------------------------------------------

def padded_len(n):
    """Smallest m >= 3n/2 with (m - n) even (``ext/FlowInvariantTransferFFTWExt.jl:128-131``)."""
    m = -(-3 * n // 2)
    return m if (m - n) % 2 == 0 else m + 1


def embed_spectrum(A, Ms):
    """fftshift-centred zero padding (``ext/FlowInvariantTransferFFTWExt.jl:134-141``)."""
    nd = A.ndim
    c = np.fft.fftshift(A)
    B = np.zeros(tuple(Ms), dtype=A.dtype)
    sl = tuple(slice((Ms[d] - A.shape[d]) // 2, (Ms[d] - A.shape[d]) // 2 + A.shape[d]) for d in range(nd))
    B[sl] = c
    return np.fft.ifftshift(B)


def truncate_spectrum(A, ns):
    """Inverse of :func:`embed_spectrum` (``ext/FlowInvariantTransferFFTWExt.jl:144-149``)."""
    nd = A.ndim
    c = np.fft.fftshift(A)
    sl = tuple(slice((A.shape[d] - ns[d]) // 2, (A.shape[d] - ns[d]) // 2 + ns[d]) for d in range(nd))
    return np.fft.ifftshift(c[sl])


def dealias_copy(f_hat, ns):
    """Copy with the 2/3-discarded modes zeroed (``ext/FlowInvariantTransferFFTWExt.jl:186-196``)."""
    keep = keep_mask(ns)
    return f_hat * keep[..., None]


def nonlinear_term(f_hat, ks, dealiasing="two_thirds", adv_hat=None):
    """N̂_i = fft(sum_j u_j d_j f_i)/Np on the resolved grid.

    * ``two_thirds`` / ``none``: restates ``_nonlinear_term_fft!``
      (``ext/FlowInvariantTransferFFTWExt.jl:61-121``): inputs and output masked by the N÷3 rule.
    * ``three_halves``: restates ``_nonlinear_term_padded_fft!`` (``:160-183``): embed on the
      padded grid, multiply there, truncate, scale ``Mtot/Ntot^2``; the derivative multiplier
      uses the N-grid ``ks`` (+N/2 at the Nyquist index)."""
    nd = len(ks)
    ns = f_hat.shape[:nd]
    M = f_hat.shape[nd]
    adv = f_hat if adv_hat is None else adv_hat
    axes = tuple(range(nd))
    Np = float(np.prod(ns))
    kc = [_kcomp(ks, d, ns) for d in range(nd)]
    out = np.zeros(ns + (M,), dtype=np.complex128)
    if dealiasing == "three_halves":
        Ms = tuple(padded_len(n) for n in ns)
        scale = float(np.prod(Ms)) / Np ** 2
        uM = [np.real(_ifftn(embed_spectrum(adv[..., j], Ms), axes=axes)) for j in range(nd)]
        for c in range(M):
            NcM = np.zeros(Ms)
            for j in range(nd):
                gMj = np.real(_ifftn(embed_spectrum(1j * kc[j] * f_hat[..., c], Ms), axes=axes))
                NcM = NcM + uM[j] * gMj
            out[..., c] = truncate_spectrum(_fftn(NcM, axes=axes), ns) * scale
        return out
    trunc = dealiasing == "two_thirds"
    if dealiasing not in ("two_thirds", "none"):
        raise ValueError(f"unknown dealiasing {dealiasing!r}")
    keep = keep_mask(ns) if trunc else np.ones(ns, dtype=bool)
    u = [np.real(_ifftn(keep * adv[..., j], axes=axes)) for j in range(nd)]
    for c in range(M):
        Nc = np.zeros(ns)
        for j in range(nd):
            Nc = Nc + u[j] * np.real(_ifftn(1j * kc[j] * keep * f_hat[..., c], axes=axes))
        Nh = _fftn(Nc, axes=axes) / Np
        out[..., c] = Nh * keep if trunc else Nh
    return out


# ---------------------------------------------------------------------------------------------
# Transfer densities
# ---------------------------------------------------------------------------------------------

def transfer_density(invariant, carrier, Nhat, ks):
    """Per-mode real transfer density. Restates ``src/Invariants.jl:40-104``:
    KE / passive scalar ``sum_c Re{conj(c_c) N_c}``; helicity ``Re{conj(ik x u) . N}`` (3D);
    enstrophy 2D ``Re{conj(w) N_w}``, 3D with ``N_w = ik x N``."""
    nd = len(ks)
    ns = carrier.shape[:nd]
    if invariant in ("ke", "scalar"):
        return np.sum(np.real(np.conj(carrier) * Nhat), axis=nd)
    k = [_kcomp(ks, d, ns) for d in range(nd)]
    if invariant == "helicity":
        if nd != 3:
            raise ValueError(f"Helicity transfer is defined in 3D only (got nd={nd}).")
        ux, uy, uz = carrier[..., 0], carrier[..., 1], carrier[..., 2]
        wx = 1j * (k[1] * uz - k[2] * uy)
        wy = 1j * (k[2] * ux - k[0] * uz)
        wz = 1j * (k[0] * uy - k[1] * ux)
        return np.real(np.conj(wx) * Nhat[..., 0] + np.conj(wy) * Nhat[..., 1] + np.conj(wz) * Nhat[..., 2])
    if invariant == "enstrophy":
        if nd == 2:
            w = 1j * (k[0] * carrier[..., 1] - k[1] * carrier[..., 0])
            Nw = 1j * (k[0] * Nhat[..., 1] - k[1] * Nhat[..., 0])
            return np.real(np.conj(w) * Nw)
        if nd == 3:
            ux, uy, uz = carrier[..., 0], carrier[..., 1], carrier[..., 2]
            Nx, Ny, Nz = Nhat[..., 0], Nhat[..., 1], Nhat[..., 2]
            wx = 1j * (k[1] * uz - k[2] * uy); wy = 1j * (k[2] * ux - k[0] * uz); wz = 1j * (k[0] * uy - k[1] * ux)
            Nwx = 1j * (k[1] * Nz - k[2] * Ny); Nwy = 1j * (k[2] * Nx - k[0] * Nz); Nwz = 1j * (k[0] * Ny - k[1] * Nx)
            return np.real(np.conj(wx) * Nwx + np.conj(wy) * Nwy + np.conj(wz) * Nwz)
        raise ValueError(f"Enstrophy transfer is defined in 2D or 3D; got nd={nd}.")
    raise ValueError(f"unknown invariant {invariant!r}")


def _bin(t, sidx, nsh):
    sel = sidx > 0
    return np.bincount(sidx[sel].ravel() - 1, weights=t[sel].ravel(), minlength=nsh)[:nsh]


# ---------------------------------------------------------------------------------------------
# Decompositions
# ---------------------------------------------------------------------------------------------

def helical_decompose(u_hat, ks):
    """Craya-Herring helical split (positive, negative). Restates
    ``_decompose_field_spectral(::HelicalDecomposition)`` (``src/Decomposition.jl:63-98``)."""
    nd = len(ks)
    if nd != 3:
        raise ValueError(f"HelicalDecomposition is defined in 3D only (got nd={nd}).")
    ns = u_hat.shape[:3]
    kx, ky, kz = np.meshgrid(*[np.asarray(k, dtype=np.float64) for k in ks], indexing="ij")
    kk = np.sqrt(kx * kx + ky * ky + kz * kz)
    nz = kk != 0
    kks = np.where(nz, kk, 1.0)
    hx, hy, hz = kx / kks, ky / kks, kz / kks
    use_z = np.abs(hz) < 0.9
    rx = np.where(use_z, 0.0, 1.0); ry = np.zeros(ns); rz = np.where(use_z, 1.0, 0.0)
    e1x = hy * rz - hz * ry; e1y = hz * rx - hx * rz; e1z = hx * ry - hy * rx
    n1 = np.sqrt(e1x ** 2 + e1y ** 2 + e1z ** 2)
    n1 = np.where(nz, n1, 1.0)
    e1x, e1y, e1z = e1x / n1, e1y / n1, e1z / n1
    e2x = hy * e1z - hz * e1y; e2y = hz * e1x - hx * e1z; e2z = hx * e1y - hy * e1x
    u1, u2, u3 = u_hat[..., 0], u_hat[..., 1], u_hat[..., 2]
    ue1 = u1 * e1x + u2 * e1y + u3 * e1z
    ue2 = u1 * e2x + u2 * e2y + u3 * e2z
    s = 1.0 / np.sqrt(2.0)
    upc = (ue1 - 1j * ue2) * s
    umc = (ue1 + 1j * ue2) * s
    up = np.zeros_like(u_hat, dtype=np.complex128)
    um = np.zeros_like(u_hat, dtype=np.complex128)
    for c, (e1c, e2c) in enumerate(((e1x, e2x), (e1y, e2y), (e1z, e2z))):
        up[..., c] = np.where(nz, upc * ((e1c + 1j * e2c) * s), 0)
        um[..., c] = np.where(nz, umc * ((e1c - 1j * e2c) * s), 0)
    return {"positive": up, "negative": um}


def toroidal_poloidal_decompose(u_hat, ks):
    """Toroidal/poloidal split (``src/Decomposition.jl:107-141``)."""
    ns = u_hat.shape[:3]
    kx, ky, kz = np.meshgrid(*[np.asarray(k, dtype=np.float64) for k in ks], indexing="ij")
    kk = np.sqrt(kx * kx + ky * ky + kz * kz)
    nz = kk != 0
    kks = np.where(nz, kk, 1.0)
    hx, hy, hz = kx / kks, ky / kks, kz / kks
    kperp = np.sqrt(kx * kx + ky * ky)
    e1x = hy * 1.0 - hz * 0.0; e1y = hz * 0.0 - hx * 1.0; e1z = hx * 0.0 - hy * 0.0
    n1 = np.sqrt(e1x ** 2 + e1y ** 2 + e1z ** 2)
    n1 = np.where(n1 > 0, n1, 1.0)
    e1x, e1y, e1z = e1x / n1, e1y / n1, e1z / n1
    e2x = hy * e1z - hz * e1y; e2y = hz * e1x - hx * e1z; e2z = hx * e1y - hy * e1x
    deg = kperp == 0
    e1x = np.where(deg, 1.0, e1x); e1y = np.where(deg, 0.0, e1y); e1z = np.where(deg, 0.0, e1z)
    e2x = np.where(deg, 0.0, e2x); e2y = np.where(deg, 1.0, e2y); e2z = np.where(deg, 0.0, e2z)
    u1, u2, u3 = u_hat[..., 0], u_hat[..., 1], u_hat[..., 2]
    c1 = u1 * e1x + u2 * e1y + u3 * e1z
    c2 = u1 * e2x + u2 * e2y + u3 * e2z
    tor = np.zeros_like(u_hat, dtype=np.complex128); pol = np.zeros_like(u_hat, dtype=np.complex128)
    for c, (a, b) in enumerate(((e1x, e2x), (e1y, e2y), (e1z, e2z))):
        tor[..., c] = np.where(nz, c1 * a, 0)
        pol[..., c] = np.where(nz, c2 * b, 0)
    return {"toroidal": tor, "poloidal": pol}


def helmholtz_decompose(u_hat, ks):
    """Rotational/divergent split as a spectral Leray projection:
    ``u_div = k (k.u)/|k|^2``, ``u_rot = u - u_div``, the mean mode kept in ``u_rot``.

    The reference delegates to the un-vendored HelmholtzDecomposition.jl
    (``ext/FlowInvariantTransferHelmholtzDecompositionExt.jl:50-104``, 2D only); this restates
    the projection that package's name and the reference tests (``test/runtests.jl:607-631``)
    describe. Parity beyond those relational tests is unpinned."""
    nd = len(ks)
    if u_hat.shape[nd] != 2 or nd != 2:
        raise ValueError("Helmholtz decomposition currently supports 2D fields only.")
    kx, ky = np.meshgrid(*[np.asarray(k, dtype=np.float64) for k in ks], indexing="ij")
    k2 = kx * kx + ky * ky
    inv = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    kd = (kx * u_hat[..., 0] + ky * u_hat[..., 1]) * inv
    div = np.stack([kx * kd, ky * kd], axis=-1)
    return {"rotational": u_hat - div, "divergent": div}


# ---------------------------------------------------------------------------------------------
# Diagnostics
# ---------------------------------------------------------------------------------------------

def spectral_flux(u_hat, ks, binning=None, dealiasing="two_thirds", invariant="ke",
                  adv_hat=None, dims=None, carrier=None):
    """(centers, T, Pi). Restates ``calculate_spectral_flux`` →
    ``_calculate_spectral_flux_with_N̂!`` (``src/SpectralFlux.jl:49-94,148-180``):
    ``T[n] = sum_{k in S_n} t(k)``, ``Pi = +cumsum(T)`` (``:176``). ``carrier`` replaces the
    density's first factor (the decomposed-component branch ``:86-91``)."""
    binning = default_binning(ks) if binning is None else binning
    nd = len(ks)
    _, edges, centers, sidx = shell_setup(ks, binning, dims)
    Nh = nonlinear_term(u_hat, ks, dealiasing, adv_hat)
    t = transfer_density(invariant, u_hat if carrier is None else carrier, Nh, ks)
    T = _bin(t, sidx, len(centers))
    return centers, T, np.cumsum(T)


def s2s_setup(u_hat, ks, binning=None, dealiasing="two_thirds", invariant="ke", adv_hat=None, dims=None):
    """Mediator-independent part of ``_shell_to_shell_fft!``
    (``ext/FlowInvariantTransferFFTWExt.jl:209-237``): shells, truncated copies and the advecting
    velocity in physical space (computed once)."""
    binning = default_binning(ks) if binning is None else binning
    nd = len(ks)
    ns = u_hat.shape[:nd]
    adv = u_hat if adv_hat is None else adv_hat
    _, edges, centers, sidx = shell_setup(ks, binning, dims)
    trunc = dealiasing == "two_thirds"
    keep = keep_mask(ns)
    st = dict(u_hat=u_hat, ks=ks, nd=nd, ns=ns, M=u_hat.shape[nd], adv=adv, edges=edges, centers=centers,
              sidx=sidx, nsh=len(centers), Np=float(np.prod(ns)), trunc=trunc,
              padded=dealiasing == "three_halves", keep=keep, invariant=invariant,
              axes=tuple(range(nd)), kc=[_kcomp(ks, d, ns) for d in range(nd)])
    st["vhat"] = u_hat * keep[..., None] if trunc else u_hat
    if not st["padded"]:
        ahat = adv * keep[..., None] if trunc else adv
        st["u_full"] = [np.real(_ifftn(ahat[..., j], axes=st["axes"])) for j in range(nd)]
    return st


def s2s_column(st, m, comps=None):
    """Column m (0-based) of T: ``ext/FlowInvariantTransferFFTWExt.jl:245-275``. ``comps``
    restricts the advected components evaluated (a bounded CPU timing sample); the column is
    then the partial sum over those components."""
    nd, ns, M, axes, kc = st["nd"], st["ns"], st["M"], st["axes"], st["kc"]
    um = st["vhat"] * (st["sidx"] == m + 1)[..., None]
    comps = range(M) if comps is None else comps
    if st["padded"]:
        Nh = nonlinear_term(um, st["ks"], "three_halves", st["adv"])
    else:
        Nh = np.zeros(ns + (M,), dtype=np.complex128)
        for c in comps:
            Nc = np.zeros(ns)
            for j in range(nd):
                Nc = Nc + st["u_full"][j] * np.real(_ifftn(1j * kc[j] * um[..., c], axes=axes))
            Nh[..., c] = _fftn(Nc, axes=axes) / st["Np"]
        if st["trunc"]:
            Nh = Nh * st["keep"][..., None]
    t = transfer_density(st["invariant"], st["u_hat"], Nh, st["ks"])
    return _bin(t, st["sidx"], st["nsh"])


def shell_to_shell(u_hat, ks, binning=None, dealiasing="two_thirds", invariant="ke",
                   adv_hat=None, dims=None, verify=True, mediators=None):
    """(centers, edges, T[n,m], net, max_asym). Restates ``_shell_to_shell_fft!``
    (``ext/FlowInvariantTransferFFTWExt.jl:209-295``): the full (2/3-truncated) velocity
    advects the band-m field taken from the truncated copy; the carrier is the untruncated
    field; no antisymmetrisation. ``mediators`` (0-based) limits the columns computed (for a
    bounded CPU timing sample); the others stay zero."""
    st = s2s_setup(u_hat, ks, binning, dealiasing, invariant, adv_hat, dims)
    nsh = st["nsh"]
    T = np.zeros((nsh, nsh))
    cols = range(nsh) if mediators is None else mediators
    for m in cols:
        T[:, m] = s2s_column(st, m)
    net = T.sum(axis=1)
    asym = float(np.max(np.abs(T + T.T))) if verify else float("nan")
    return st["centers"], st["edges"], T, net, asym


def partial_fluxes(u_hat, ks, decomposition="helical", binning=None, dealiasing="two_thirds",
                   dims=None, invariant="ke"):
    """Per-channel partial fluxes ``T^{sk,sp,sq}(k) = Re{conj(u_sk) . [(u_sp . grad) u_sq]}``.

    Restates ``calculate_partial_fluxes`` (``src/SpectralFlux.jl:240-285``), which hard-codes the
    kinetic-energy density at ``:277``; ``invariant="helicity"`` swaps the density at that line
    (the helical channels of the helicity flux have no reference implementation)."""
    binning = default_binning(ks) if binning is None else binning
    if decomposition == "helical":
        comps = helical_decompose(u_hat, ks)
    elif decomposition == "helmholtz":
        comps = helmholtz_decompose(u_hat, ks)
    elif decomposition == "toroidal_poloidal":
        comps = toroidal_poloidal_decompose(u_hat, ks)
    else:
        raise ValueError(decomposition)
    names = list(comps.keys())
    _, edges, centers, sidx = shell_setup(ks, binning, dims)
    nsh = len(centers)
    chans = {}
    for sp in names:
        for sq in names:
            Nh = nonlinear_term(comps[sq], ks, dealiasing, comps[sp])
            for sk in names:
                t = transfer_density(invariant, comps[sk], Nh, ks)
                T = _bin(t, sidx, nsh)
                chans[(sk, sp, sq)] = (T, np.cumsum(T))
    total_T = sum(v[0] for v in chans.values())
    total_P = sum(v[1] for v in chans.values())
    return chans, (total_T, total_P), centers


def mode_to_mode(u_hat, ks, dealiasing="two_thirds", invariant="ke", adv_hat=None):
    """(net, S) with ``S[k..., p...]``. Restates the per-giver loop of
    ``calculate_mode_to_mode_transfer`` (``src/ScaleToScale/ScaleToScaleTransfer.jl:49-91``).
    O(N_modes) nonlinear terms: use for small grids only."""
    nd = len(ks)
    ns = u_hat.shape[:nd]
    M = u_hat.shape[nd]
    adv = u_hat if adv_hat is None else adv_hat
    S = np.zeros(ns + ns)
    for p in np.ndindex(*ns):
        up = np.zeros_like(u_hat)
        up[p] = u_hat[p]
        Nh = nonlinear_term(up, ks, dealiasing, adv)
        S[(Ellipsis,) + p] = transfer_density(invariant, u_hat, Nh, ks)
    net = S.reshape(int(np.prod(ns)), -1).sum(axis=1).reshape(ns)
    return net, S


def _effective_carrier(invariant, carrier, ks):
    """C with t(k) = sum_c Re{conj(C_c(k)) N_c(k)} for every invariant (densities are linear in N).
    KE/scalar: C = u; helicity: C = ik x u; enstrophy 2D: C = w (i k_y, -i k_x);
    enstrophy 3D: C = ik x (ik x u)."""
    nd = len(ks)
    ns = carrier.shape[:nd]
    if invariant in ("ke", "scalar"):
        return carrier
    k = [_kcomp(ks, d, ns) for d in range(nd)]
    def curl(v):
        return np.stack([1j * (k[1] * v[..., 2] - k[2] * v[..., 1]),
                         1j * (k[2] * v[..., 0] - k[0] * v[..., 2]),
                         1j * (k[0] * v[..., 1] - k[1] * v[..., 0])], axis=-1)
    if invariant == "helicity":
        return curl(carrier)
    if invariant == "enstrophy":
        if nd == 2:
            w = 1j * (k[0] * carrier[..., 1] - k[1] * carrier[..., 0])
            return np.stack([w * (1j * k[1]), w * (-1j * k[0])], axis=-1)
        return curl(curl(carrier))
    raise ValueError(invariant)


def mode_to_mode_triad(u_hat, ks, dealiasing="two_thirds", invariant="ke", adv_hat=None,
                       chunk=256):
    """Closed form of the per-giver loop above (same S up to FP64 rounding):

        N_p(k) = keep(k)/(2 Np^2) sum_j [A_j(k-p) i k_j(p) f(p) + A_j(k+p) conj(i k_j(p) f(p))]
        S(k|p) = sum_c Re{conj(C_c(k)) N_p,c(k)}

    with ``A = Herm(keep . u_adv)`` (what ``real(ifft)`` keeps), ``f = keep . u`` and indices
    ``k -/+ p`` taken mod N (aliasing wraps exactly as the FFT does). Derived from
    ``_nonlinear_term_fft!`` (``ext/FlowInvariantTransferFFTWExt.jl:61-121``) applied to a
    single-mode field; checked against :func:`mode_to_mode` in the tests."""
    if dealiasing == "three_halves":
        raise ValueError("closed-form triads cover the two_thirds / none paths")
    nd = len(ks)
    ns = u_hat.shape[:nd]
    M = u_hat.shape[nd]
    adv = u_hat if adv_hat is None else adv_hat
    Nm = int(np.prod(ns))
    keep = keep_mask(ns) if dealiasing == "two_thirds" else np.ones(ns, dtype=bool)
    f = (u_hat * keep[..., None])
    a = adv[..., :nd] * keep[..., None]
    neg = tuple(np.arange(0, -n, -1) % n for n in ns)
    a_neg = a[np.ix_(*neg)] if nd > 1 else a[neg[0]]
    A = 0.5 * (a + np.conj(a_neg))
    C = _effective_carrier(invariant, u_hat, ks)
    grids = np.meshgrid(*[np.arange(n) for n in ns], indexing="ij")
    kidx = [g.ravel(order="F") for g in grids]          # column-major flattening (Julia order)
    kvec = [np.asarray(ks[d], dtype=np.float64)[kidx[d]] for d in range(nd)]
    Af = [A[..., j].ravel(order="F") for j in range(nd)]
    ff = [f[..., c].ravel(order="F") for c in range(M)]
    Cf = [C[..., c].ravel(order="F") for c in range(M)]
    keepf = keep.ravel(order="F")
    strides = [int(np.prod(ns[:d])) for d in range(nd)]

    def lin(idx):
        return sum(idx[d] * strides[d] for d in range(nd))

    S = np.zeros((Nm, Nm))
    for p0 in range(0, Nm, chunk):
        p = np.arange(p0, min(Nm, p0 + chunk))
        kminus = lin([(kidx[d][:, None] - kidx[d][p][None, :]) % ns[d] for d in range(nd)])
        kplus = lin([(kidx[d][:, None] + kidx[d][p][None, :]) % ns[d] for d in range(nd)])
        a1 = sum(Af[j][kminus] * kvec[j][p][None, :] for j in range(nd))
        a2 = sum(Af[j][kplus] * kvec[j][p][None, :] for j in range(nd))
        cf = sum(np.conj(Cf[c])[:, None] * ff[c][p][None, :] for c in range(M))
        cfc = sum(np.conj(Cf[c])[:, None] * np.conj(ff[c][p])[None, :] for c in range(M))
        val = np.real(1j * a1 * cf - 1j * a2 * cfc) * (keepf[:, None] / (2.0 * Nm * Nm))
        S[:, p] = val
    net = S.sum(axis=1).reshape(ns, order="F")
    return net, S.reshape(ns + ns, order="F")


# ---------------------------------------------------------------------------------------------
# Coarse-graining flux (restated; the reference delegates to an un-vendored 2D package)
# ---------------------------------------------------------------------------------------------

def filter_response(kind, k, ell):
    """Spectral filter responses (``src/Filters.jl:19-26``)."""
    if kind == "gaussian":
        return np.exp(-(k ** 2) * ell ** 2 / 24)
    if kind == "sharp":
        return np.where(np.abs(k) < np.pi / ell, 1.0, 0.0)
    if kind == "tophat":
        return np.sinc(k * ell / (2 * np.pi))
    raise ValueError(kind)


def coarse_graining_flux(u_phys, ks, ell, kind="gaussian"):
    """Pi_ell(x) = -tau_ij S_ij with tau_ij = bar(u_i u_j) - bar(u_i) bar(u_j) and
    S_ij = (d_j bar(u_i) + d_i bar(u_j))/2, filters applied spectrally with ``filter_response``.

    Restated from the formula in ``THEORY.md:64-71,210-217`` and ``src/Filters.jl:22-23``; the
    reference computes it through the un-vendored CoarseGrainingEnergyFluxes.jl in 2D only
    (``ext/FlowInvariantTransferCGEFExt.jl:42``), so this n-D form is unpinned."""
    nd = len(ks)
    ns = u_phys.shape[:nd]
    axes = tuple(range(nd))
    kc = [_kcomp(ks, d, ns) for d in range(nd)]
    kmag = np.sqrt(sum(k * k for k in kc))
    G = filter_response(kind, kmag, ell)

    def filt(f):
        return np.real(_ifftn(G * _fftn(f, axes=axes), axes=axes))

    ub = [filt(u_phys[..., i]) for i in range(nd)]
    ubh = [_fftn(ub[i], axes=axes) for i in range(nd)]
    grad = [[np.real(_ifftn(1j * kc[j] * ubh[i], axes=axes)) for j in range(nd)] for i in range(nd)]
    Pi = np.zeros(ns)
    for i in range(nd):
        for j in range(nd):
            tau = filt(u_phys[..., i] * u_phys[..., j]) - ub[i] * ub[j]
            Sij = 0.5 * (grad[i][j] + grad[j][i])
            Pi = Pi - tau * Sij
    return Pi


# ---------------------------------------------------------------------------------------------
# Smooth band-to-band transfer
# ---------------------------------------------------------------------------------------------

def band_weights(centers, logwidth, kcoord):
    """Renormalised log-Gaussian band weights ``w_n(kappa)`` (``src/BandTransfer.jl:24-46``):
    ``exp(-(ln(kappa/c_n))^2 / (2 sigma^2))`` divided by their sum over bands; zero where
    ``kappa <= 0``."""
    kappa = np.asarray(kcoord, dtype=np.float64)
    pos = kappa > 0
    kp = np.where(pos, kappa, 1.0)
    W = []
    for c in centers:   # r = ln(kappa / c), exp(-r^2 / (2 sigma sigma)), in the reference's order (:35-36)
        r = np.log(kp / float(c))
        W.append(np.where(pos, np.exp(-(r * r) / (2.0 * logwidth * logwidth)), 0.0))
    W = np.stack(W)
    s = W.sum(axis=0)
    return np.where(s > 0, W / np.where(s > 0, s, 1.0), 0.0)


def band_to_band(u_hat, ks, centers, logwidth=0.6, dealiasing="two_thirds", invariant="ke", adv_hat=None,
                 dims=None):
    """(centers, T, net, max_asym). Restates ``calculate_band_to_band_transfer``
    (``src/BandTransfer.jl:71-113``): for each band m the nonlinear term of ``w_m * f`` advected by
    the full velocity, its transfer density against the full field, weighted by ``w_n``."""
    nd = len(ks)
    ns = u_hat.shape[:nd]
    adv = u_hat if adv_hat is None else adv_hat
    W = band_weights(centers, logwidth, shell_coordinate(ks, dims))
    nb = len(centers)
    T = np.zeros((nb, nb))
    for m in range(nb):
        fm = u_hat * W[m][..., None]
        Nh = nonlinear_term(fm, ks, dealiasing, adv)
        d = transfer_density(invariant, u_hat, Nh, ks)
        for n in range(nb):
            T[n, m] = float(np.sum(W[n] * d))
    net = T.sum(axis=1)
    asym = float(np.max(np.abs(T + T.T)))
    return np.asarray(centers, dtype=np.float64), T, net, asym
