"""Direct-sum restatement of the reference's DirectSumBackend (TEST ORACLE ONLY).

Restates ``_compute_nonlinear_term_direct!`` (``src/NonlinearTerm.jl:160-265``): explicit
O(N^{2D}) inverse/forward DFT sums with the same phase convention, the 2/3 input skip and the
output zeroing. Each sum is written as a dense DFT-matrix contraction (the same arithmetic as
the reference's loops, in a different summation order). Used to pin the FFT restatement in
``fit_oracle`` on small grids (N <= 16), as the reference's own tests do
(``test/runtests.jl:151-172,412-438``).
"""
from __future__ import annotations

import numpy as np

from .fit_oracle import keep_mask, transfer_density, shell_setup, default_binning


def _dft_matrix(N, sign):
    x = np.arange(N) / N
    kidx = np.arange(N)
    km = np.where(kidx <= N // 2, kidx, kidx - N)
    return np.exp(sign * 1j * 2 * np.pi * np.outer(km, x))   # [k, x]


def _idft(a, nd):
    out = a
    for d in range(nd):
        E = _dft_matrix(a.shape[d], +1)        # sum_k a(k) e^{+i 2pi km x}
        out = np.moveaxis(np.tensordot(E.T, np.moveaxis(out, d, 0), axes=(1, 0)), 0, d)
    return out / np.prod(a.shape[:nd])


def _dft(a, nd):
    out = a
    for d in range(nd):
        E = _dft_matrix(a.shape[d], -1)
        out = np.moveaxis(np.tensordot(E, np.moveaxis(out, d, 0), axes=(1, 0)), 0, d)
    return out / np.prod(a.shape[:nd])


def nonlinear_term_direct(f_hat, ks, truncate=True, adv_hat=None):
    """``_compute_nonlinear_term_direct!`` (``src/NonlinearTerm.jl:160-265``)."""
    nd = len(ks)
    ns = f_hat.shape[:nd]
    M = f_hat.shape[nd]
    adv = f_hat if adv_hat is None else adv_hat
    keep = keep_mask(ns) if truncate else np.ones(ns, dtype=bool)
    u = [np.real(_idft(adv[..., j] * keep, nd)) for j in range(nd)]
    out = np.zeros(ns + (M,), dtype=np.complex128)
    for c in range(M):
        Nc = np.zeros(ns)
        for j in range(nd):
            shape = [1] * nd
            shape[j] = ns[j]
            kj = np.asarray(ks[j]).reshape(shape)
            Nc = Nc + u[j] * np.real(_idft(1j * kj * f_hat[..., c] * keep, nd))
        out[..., c] = _dft(Nc.astype(np.complex128), nd)
    if truncate:
        out = out * keep[..., None]
    return out


def shell_to_shell_direct(u_hat, ks, binning=None, truncate=True, invariant="ke", adv_hat=None,
                          dims=None):
    """``_calculate_shell_to_shell_direct!`` (``src/ShellToShell/ShellToShellTransfer.jl:176-248``):
    mediator taken from the untruncated field (the direct term truncates its inputs itself)."""
    binning = default_binning(ks) if binning is None else binning
    nd = len(ks)
    _, edges, centers, sidx = shell_setup(ks, binning, dims)
    nsh = len(centers)
    T = np.zeros((nsh, nsh))
    for m in range(nsh):
        um = u_hat * (sidx == m + 1)[..., None]
        Nh = nonlinear_term_direct(um, ks, truncate, u_hat if adv_hat is None else adv_hat)
        t = transfer_density(invariant, u_hat, Nh, ks)
        for n in range(nsh):
            T[n, m] = t[sidx == n + 1].sum()
    net = T.sum(axis=1)
    return centers, edges, T, net, float(np.max(np.abs(T + T.T)))
