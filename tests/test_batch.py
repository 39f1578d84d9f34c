"""Uneven batch (many spectral-flux instances as one CUDA graph launch) and the transform-pass
autotuner, against the oracle's spectral flux per instance."""
import numpy as np
import pytest

import oracle as O
from fields import e_config1, e_scalar, spectrum_field

import fit_gb300 as F

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _tuner_off_after():
    yield
    F.autotune_enable(False)


def _instances(seed=0):
    """Eight uneven instances: 2D and 3D, sizes 2^n and 3*2^n, kinetic energy and passive scalar,
    isotropic / perpendicular / parallel shells."""
    shapes = [(24, 24), (32, 32), (48, 48), (64, 64), (16, 16, 16), (12, 12, 12), (24, 24, 24), (16, 16, 16)]
    out = []
    for i, ns in enumerate(shapes):
        nd = len(ns)
        ks = O.wavenumber_grid(ns, (2 * np.pi,) * nd)
        u = spectrum_field(ns, e_config1, seed=seed + 10 * i, project=True)[0]
        geo = [F.IsotropicShells(), F.PerpendicularShells(), F.ParallelShells(dims=(nd,))][i % 3]
        spec = {"velocity_hat": u, "ks": ks, "geometry": geo, "binning": F.LinearBinning(1.0)}
        if i % 2:
            spec["scalar_hat"] = spectrum_field(ns, e_scalar, seed=seed + 10 * i + 1, project=False, ncomp=1)[0]
        out.append(spec)
    return out


def _oracle(spec):
    ks = spec["ks"]
    geo = spec["geometry"]
    dims = None if geo.dims is None else tuple(geo.dims)
    if "scalar_hat" in spec:
        _, T, Pi = O.spectral_flux(spec["scalar_hat"], ks, ("linear", 1.0), "two_thirds", "scalar",
                                   adv_hat=spec["velocity_hat"], dims=dims)
    else:
        _, T, Pi = O.spectral_flux(spec["velocity_hat"], ks, ("linear", 1.0), "two_thirds", "ke", dims=dims)
    return T, Pi


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("prec,tol", [(64, 1e-11), (32, 2e-5)])
def test_batch_matches_oracle(prec, tol):
    inst = _instances()
    b = F.SpectralFluxBatch(inst, precision=prec, n_branches=3, autotune=True)
    b.run()                      # eager: allocation + autotuning
    r_eager = b.results()
    l0 = F.launch_count()
    b.run()                      # capture + one graph launch
    b.run()                      # graph launch
    r_graph = b.results()
    info = b.info()
    assert info["state"] == 2 and info["instances"] == len(inst) and info["graph_kernels"] > len(inst)
    assert F.launch_count() - l0 == 2 * info["graph_kernels"]
    for spec, re, rg in zip(inst, r_eager, r_graph):
        T, Pi = _oracle(spec)
        assert _rel(re.transfer_spectrum, T) <= tol
        assert _rel(rg.transfer_spectrum, T) <= tol
        assert _rel(rg.flux, Pi) <= tol * 10
        assert _rel(rg.transfer_spectrum, re.transfer_spectrum) <= 1e-12
    b.close()


def test_batch_without_autotune_and_single_branch():
    inst = _instances(seed=5)[:4]
    F.autotune_clear()
    r = F.calculate_spectral_flux_batch(inst, precision=64, n_branches=1, autotune=False)
    assert F.autotune_summary()["entries"] == 0
    for spec, ri in zip(inst, r):
        T, _ = _oracle(spec)
        assert _rel(ri.transfer_spectrum, T) <= 1e-11


def test_autotune_table():
    F.autotune_clear()
    inst = _instances(seed=7)
    F.calculate_spectral_flux_batch(inst, precision=32, n_branches=2, autotune=True)
    s = F.autotune_summary()
    assert s["entries"] > 0 and len(s["table"]) == s["entries"]
    for e in s["table"]:
        assert e["ms_best"] <= e["ms_default"] * 1.0001 + 1e-6
        if e["engine"] == "runtime":
            assert e["C"] >= 1 and e["C"] & (e["C"] - 1) == 0 and e["ept"] in (8, 16)
    F.autotune_enable(False)


def test_batch_errors():
    ns = (16, 16)
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 2)
    u = spectrum_field(ns, e_config1, seed=1)[0]
    with pytest.raises(ValueError):
        F.SpectralFluxBatch([{"velocity_hat": u, "ks": ks, "invariant": F.Helicity()}])
    b = F.SpectralFluxBatch([{"velocity_hat": u, "ks": ks}], precision=64)
    b.run()
    T, _ = _oracle({"velocity_hat": u, "ks": ks, "geometry": F.IsotropicShells()})
    assert _rel(b.results()[0].transfer_spectrum, T) <= 1e-11
    b.run_eager()
    assert _rel(b.results()[0].transfer_spectrum, T) <= 1e-11
    b.close()
