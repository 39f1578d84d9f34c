"""Seeded synthetic spectral fields shared by the tests, the golden-vector script and the bench.

The constructions mirror the reference test suite (``test/runtests.jl``): a 2D solenoidal field
from a random streamfunction (``:184-191``), a 3D solenoidal field ``û = i k × Â`` from complex
noise (``:509-515``; NOT Hermitian), and the spectrum-shaped Hermitian solenoidal fields of the
benchmark configurations (random-phase real noise, FFT, amplitude ``sqrt(E(|k|)/|k|^{nd-1})``,
Leray projection, DC removed; scalar fields skip the projection).
"""
from __future__ import annotations

import numpy as np


def kgrid(ns, Ls=None):
    Ls = Ls or tuple(2 * np.pi for _ in ns)
    out = []
    for N, L in zip(ns, Ls):
        idx = np.arange(N)
        out.append(np.where(idx <= N // 2, idx, idx - N).astype(np.float64) * (2 * np.pi / L))
    return tuple(out)


def solenoidal_2d(N, seed):
    rng = np.random.default_rng(seed)
    ks = kgrid((N, N))
    kx, ky = np.meshgrid(*ks, indexing="ij")
    psih = np.fft.fft2(rng.standard_normal((N, N))) / N ** 2
    u = np.stack([1j * ky * psih, -1j * kx * psih], axis=-1)
    return np.asfortranarray(u), ks


def scalar_2d(N, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray((np.fft.fft2(rng.standard_normal((N, N))) / N ** 2)[..., None])


def curl_noise_3d(N, seed, hermitian=False):
    """û = i k × Â with complex-normal Â (the reference's 3D test field, non-Hermitian), or
    with Â = fft(real noise) when ``hermitian``."""
    rng = np.random.default_rng(seed)
    ks = kgrid((N, N, N))
    kx, ky, kz = np.meshgrid(*ks, indexing="ij")
    if hermitian:
        A = np.fft.fftn(rng.standard_normal((N, N, N, 3)), axes=(0, 1, 2)) / N ** 3
    else:
        A = rng.standard_normal((N, N, N, 3)) + 1j * rng.standard_normal((N, N, N, 3))
    u = np.stack([1j * (ky * A[..., 2] - kz * A[..., 1]),
                  1j * (kz * A[..., 0] - kx * A[..., 2]),
                  1j * (kx * A[..., 1] - ky * A[..., 0])], axis=-1)
    return np.asfortranarray(u), ks


def spectrum_field(ns, spectrum, seed, project=True, ncomp=None, dtype=np.complex128):
    """Hermitian random-phase field with shell energy spectrum ``spectrum(|k|)``.

    ``û = fft(u)/Np`` of real Gaussian noise, each mode scaled by ``sqrt(E(|k|)/|k|^{nd-1})``,
    Leray-projected (``project``) and with the mean mode removed."""
    nd = len(ns)
    ncomp = nd if ncomp is None else ncomp
    rng = np.random.default_rng(seed)
    ks = kgrid(ns)
    kk = np.meshgrid(*ks, indexing="ij")
    kmag = np.sqrt(sum(k * k for k in kk))
    Np = float(np.prod(ns))
    out = np.empty(tuple(ns) + (ncomp,), dtype=np.complex128, order="F")
    with np.errstate(divide="ignore", invalid="ignore"):
        amp = np.where(kmag > 0, np.sqrt(spectrum(kmag) / np.where(kmag > 0, kmag, 1.0) ** (nd - 1)), 0.0)
    for c in range(ncomp):
        out[..., c] = np.fft.fftn(rng.standard_normal(tuple(ns)), axes=tuple(range(nd))) / Np * amp
    if project and ncomp == nd:
        k2 = np.where(kmag > 0, kmag * kmag, 1.0)
        div = sum(kk[d] * out[..., d] for d in range(nd)) / k2
        for d in range(nd):
            out[..., d] -= kk[d] * div
    out[(0,) * nd] = 0
    return np.asfortranarray(out.astype(dtype)), ks


def e_config1(k):
    """E(k) ∝ k^4 exp(-2 (k/4)^2): the 64² spectral-flux workload."""
    return k ** 4 * np.exp(-2 * (k / 4.0) ** 2)


def e_config2(k):
    """E(k) ∝ k^4 exp(-2 (k/8)^2): the 3D shell-to-shell / mode-to-mode workloads."""
    return k ** 4 * np.exp(-2 * (k / 8.0) ** 2)


def e_kolmogorov(k):
    """k^{-5/3} on 4 <= k <= 170, (k/4)^4 4^{-5/3} below 4, zero above 170."""
    return np.where(k < 4, (k / 4.0) ** 4 * 4.0 ** (-5 / 3),
                    np.where(k <= 170, np.maximum(k, 1e-30) ** (-5 / 3), 0.0))


def e_scalar(k):
    """Scalar variance spectrum ∝ k^2 exp(-(k/6)^2)."""
    return k ** 2 * np.exp(-(k / 6.0) ** 2)
