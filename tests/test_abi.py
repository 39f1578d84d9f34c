"""CPU-side checks of the C ABI: the shared library builds, loads and exports every entry point
that include/fit_gb300.h declares; host-side shell geometry matches the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

import fit_gb300 as F
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "fit_gb300.h")).read()
    return sorted(set(re.findall(r"\b(fit_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = F._lib.load()
    names = declared_symbols()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    assert set(F._lib.EXPORTS) <= set(names)


def test_last_error_is_callable_without_gpu():
    lib = F._lib.load()
    assert isinstance(lib.fit_last_error(), bytes)


@pytest.mark.parametrize("ns", [(64, 64), (512, 512, 512), (8,), (24, 24), (16, 16, 16)])
@pytest.mark.parametrize("binning", [("linear", 1.0), ("dyadic", 2.0), ("linear", 14.0), ("log", 1.5, 1.7)])
def test_host_shell_edges_match_oracle(ns, binning):
    ks = F.wavenumber_grid(ns, tuple(2 * np.pi for _ in ns))
    kc = np.sqrt(sum(np.max(np.asarray(k) ** 2) for k in ks))
    okm = float(O.shell_coordinate(ks).max()) if np.prod(ns) <= 70000 else kc
    assert float(F.kmax(ks)) == okm
    b = {"linear": lambda: F.LinearBinning(binning[1]), "dyadic": lambda: F.DyadicBinning(binning[1]),
         "log": lambda: F.LogarithmicBinning(binning[1], binning[2])}[binning[0]]()
    try:
        e = O.shell_edges(binning, okm)
    except ValueError:
        with pytest.raises(ValueError):
            F.shell_edges(b, F.kmax(ks))
        return
    assert np.array_equal(F.shell_edges(b, F.kmax(ks)), e)
    assert np.array_equal(F.shell_centers(b, F.kmax(ks)), O.shell_centers(binning, okm))


def test_float32_wavenumbers_and_edges():
    ks = F.wavenumber_grid((8, 8), (np.float32(2 * np.pi), np.float32(2 * np.pi)))
    assert ks[0].dtype == np.float32
    km = F.kmax(ks)
    assert isinstance(km, np.float32)
    e = F.shell_edges(F.LinearBinning(np.float32(2 * np.pi) / 8), km)
    assert e.dtype == np.float32


def test_geometry_dims_validation():
    with pytest.raises(ValueError):
        F.dims_mask(F.ParallelShells(), 2)
    assert F.dims_mask(F.PerpendicularShells(), 3) == 0b011
    assert F.dims_mask(F.IsotropicShells(), 3) == 0b111
