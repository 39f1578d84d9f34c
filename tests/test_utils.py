"""The reference's Utils testsets (``test/runtests.jl:25-55``) through this package's host
utilities: FFTW-order wavenumbers, the |k| grid and the 2/3 keep mask."""
import numpy as np

import fit_gb300 as F


def test_wavenumber_grid_and_magnitude():      # runtests.jl:25-42
    N, L = 8, 2 * np.pi
    ks = F.wavenumber_grid((N, N), (L, L))
    assert len(ks) == 2 and len(ks[0]) == N
    dk = 2 * np.pi / L
    assert abs(ks[0][0]) < 1e-14 and abs(ks[0][1] - dk) < 1e-14 and abs(ks[0][N - 1] + dk) < 1e-14
    k_mag = F.wavenumber_magnitude_grid(ks)
    assert k_mag.shape == (N, N) and np.all(k_mag >= 0) and k_mag[0, 0] == 0.0
    ks3 = F.wavenumber_grid((6, 4, 10), (2 * np.pi, 3.0, 5.0))
    m3 = F.wavenumber_magnitude_grid(ks3)
    kx, ky, kz = np.meshgrid(*ks3, indexing="ij")
    assert m3.shape == (6, 4, 10) and np.array_equal(m3, np.sqrt(((0.0 + kx * kx) + ky * ky) + kz * kz))
    ks32 = F.wavenumber_grid((8, 8), (np.float32(2 * np.pi),) * 2)
    assert F.wavenumber_magnitude_grid(ks32).dtype == np.float32


def test_dealiasing_mask():                     # runtests.jl:44-54
    N = 12
    mask = F.dealiasing_mask((N, N))
    assert mask.shape == (N, N)
    assert mask[0, 0] and mask[1, 0] and not mask[4, 0]
    # the floating-point threshold: N = 64 keeps |k| <= 21 (64/3 = 21.33), N = 8 keeps |k| <= 2
    assert F.dealiasing_mask((64,)).sum() == 2 * 21 + 1
    assert F.dealiasing_mask((8,)).sum() == 2 * 2 + 1
    half = F.dealiasing_mask((8, 6), rule="half")
    assert half.sum() == 7 * 5                   # |k| < N/2 on both axes: Nyquist dropped
    out = np.zeros((N, N, N), dtype=bool)
    assert F.dealiasing_mask((N, N, N), out=out) is out and np.array_equal(out, F.dealiasing_mask((N, N, N)))
