"""Host-side shell geometry: wavenumber vectors, shell edges and centres.

These mirror ``src/Utils.jl:51-63`` and ``src/ShellBinning.jl:19-116`` exactly (they are tiny
and feed the device kernels as explicit edge lists). The per-mode coordinate and shell index
themselves are computed on the GPU (``fit_assign_shells``), in the same FP64 (or Float32)
operation order as the reference.
"""
from __future__ import annotations

import math

import numpy as np

from .types import (CustomBinning, DyadicBinning, LinearBinning, LogarithmicBinning, ShellMagnitude)


def wavenumber_grid(ns, Ls):
    """FFTW-order wavenumbers with +N/2 at the Nyquist index (``src/Utils.jl:51-63``); the element
    type follows ``Ls`` (Float32 lengths give Float32 wavenumbers)."""
    f32 = all(isinstance(L, np.float32) for L in Ls)
    ft = np.float32 if f32 else np.float64
    out = []
    for N, L in zip(ns, Ls):
        dk = ft(2 * np.pi) / ft(L)
        idx = np.arange(N)
        km = np.where(idx <= N // 2, idx, idx - N).astype(ft)
        out.append((km * dk).astype(ft))
    return tuple(out)


def wavenumber_magnitude_grid(ks):
    """|k| at every point of the grid spanned by ``ks`` (``src/Utils.jl:76-88``): an array of shape
    (len(ks[0]), ..., len(ks[D-1])) in the promoted element type of ``ks`` (Float32 wavenumbers give
    Float32 magnitudes), the squares summed in dimension order from zero and the square root taken
    once, as the reference does."""
    ks = [np.asarray(k) for k in ks]
    ft = np.result_type(*[k.dtype for k in ks])
    D = len(ks)
    s = np.zeros(tuple(len(k) for k in ks), dtype=ft)
    for d, k in enumerate(ks):
        shape = [1] * D
        shape[d] = len(k)
        kk = k.astype(ft, copy=False).reshape(shape)
        s = s + kk * kk
    return np.sqrt(s)


def dealiasing_mask(ns, rule="twothirds", out=None):
    """Keep/discard mask of grid shape ``ns`` (``dealiasing_mask`` / ``dealiasing_mask!``,
    ``src/Utils.jl:110-138``): True where every axis keeps its mode, i.e. the FFTW-order index's
    ``|k_d| = min(i, N_d - i)`` is below ``N_d * threshold``; threshold 1/3 for ``rule="twothirds"``,
    else 1/2. The threshold is the reference's floating-point one (``N/3``, so N = 64 keeps
    ``|k| <= 21``), not the integer ``N div 3`` cut of the nonlinear term's dealiasing. With ``out``
    (a boolean array of shape ``ns``) the mask is written there and ``out`` returned, as the
    in-place form does."""
    ns = tuple(int(n) for n in ns)
    threshold = 1.0 / 3.0 if rule == "twothirds" else 0.5
    keep = np.ones(ns, dtype=bool)
    for d, N in enumerate(ns):
        idx = np.arange(N)
        kabs = np.where(idx <= N // 2, idx, N - idx)
        shape = [1] * len(ns)
        shape[d] = N
        keep &= (kabs < N * threshold).reshape(shape)
    if out is None:
        return keep
    if out.shape != ns:
        raise ValueError(f"mask has shape {out.shape}; expected {ns}")
    out[...] = keep
    return out


def dims_of(geometry, nd):
    dims = tuple(range(1, nd + 1)) if geometry is None or geometry.dims is None else tuple(geometry.dims)
    if not all(1 <= d <= nd for d in dims):
        raise ValueError(f"ShellMagnitude dims={dims} out of range for nd={nd} spatial dimensions.")
    return dims


def dims_mask(geometry, nd) -> int:
    m = 0
    for d in dims_of(geometry, nd):
        m |= 1 << (d - 1)
    return m


def coord_is_f32(ks) -> bool:
    return np.asarray(ks[0]).dtype == np.float32


def kmax(ks, geometry=None):
    """Maximum shell coordinate over all modes: sum_d max_i k_d[i]^2 accumulated in dims order
    (addition of non-negative terms is monotone, so the corner attains the maximum)."""
    nd = len(ks)
    ft = np.float32 if coord_is_f32(ks) else np.float64
    s = ft(0)
    for d in dims_of(geometry, nd):
        k = np.asarray(ks[d - 1]).astype(ft)
        s = ft(s + np.max(k * k))
    return ft(np.sqrt(s))


def _julia_range(start, step, stop):
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


def shell_edges(binning, k_max):
    """``src/ShellBinning.jl:50-79``. Float32 ``k_max`` gives Float32 edges (as Julia does)."""
    f32 = isinstance(k_max, np.float32)
    km = float(k_max)
    if isinstance(binning, LinearBinning):
        if not binning.dk > 0:
            raise ValueError("LinearBinning: Δk must be positive.")
        if not km > 0:
            raise ValueError("k_max must be positive.")
        dk = float(np.float32(binning.dk)) if f32 else float(binning.dk)
        e = _julia_range(0.0, dk, km)
        if f32:
            e = e.astype(np.float32).astype(np.float64)
        e = list(e)
        if e[-1] < km:
            e.append(km)
        out = np.asarray(e, dtype=np.float64)
    elif isinstance(binning, (LogarithmicBinning, DyadicBinning)):
        k0 = float(binning.k0)
        lam = 2.0 if isinstance(binning, DyadicBinning) else float(binning.lam)
        if not k0 > 0:
            raise ValueError("LogarithmicBinning: k₀ must be positive.")
        if not lam > 1:
            raise ValueError("LogarithmicBinning: λ must be > 1.")
        if not km >= k0:
            raise ValueError("k_max must be >= k₀.")
        n_max = int(math.floor(math.log(km / k0) / math.log(lam)))
        e = [k0 * lam ** n for n in range(0, n_max + 2)]
        while len(e) > 2 and e[-2] > km:
            e.pop()
        out = np.asarray(e, dtype=np.float64)
    elif isinstance(binning, CustomBinning):
        out = np.asarray(binning.edges, dtype=np.float64)
        if not np.all(np.diff(out) >= 0):
            raise ValueError("CustomBinning: edges must be monotonically increasing.")
    else:
        raise ValueError(f"unknown binning {binning!r}")
    return out.astype(np.float32) if f32 else out


def shell_centers(binning, k_max):
    """Geometric mean for Log/Dyadic, arithmetic otherwise (``src/ShellBinning.jl:91-106``)."""
    e = shell_edges(binning, k_max)
    if len(e) - 1 <= 0:
        raise ValueError(f"No shells within k_max={k_max} for this binning.")
    if isinstance(binning, (LogarithmicBinning, DyadicBinning)):
        return np.sqrt(e[:-1] * e[1:])
    return (e[:-1] + e[1:]) / 2


def n_shells(binning, k_max):
    return len(shell_edges(binning, k_max)) - 1


def default_binning(ks):
    """``LinearBinning(min |k| > 0)`` (``src/SpectralFlux.jl:301-313``)."""
    m = math.inf
    for k in ks:
        a = np.abs(np.asarray(k, dtype=np.float64))
        a = a[a > 0]
        if a.size:
            m = min(m, float(a.min()))
    return LinearBinning(m if math.isfinite(m) else 1.0)
