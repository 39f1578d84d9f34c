"""The ctypes declarations of the Python binding agree with the C header: every function declared in
include/fit_gb300.h that the binding types has the same number of parameters (no GPU needed)."""
import os
import re

import fit_gb300 as F

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_params():
    src = open(os.path.join(ROOT, "include", "fit_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    out = {}
    for m in re.finditer(r"\b(fit_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src):
        name, params = m.group(1), m.group(2).strip()
        out[name] = 0 if params in ("", "void") else len([p for p in params.split(",") if p.strip()])
    return out


class _Fn:
    argtypes = None
    restype = None


class _FakeLib:
    def __init__(self):
        self.fns = {}

    def __getattr__(self, name):
        if name.startswith("fit_"):
            return self.fns.setdefault(name, _Fn())
        raise AttributeError(name)


def test_binding_matches_header():
    hdr = _header_params()
    assert len(hdr) >= len(F._lib.EXPORTS)
    for name in F._lib.EXPORTS:
        assert name in hdr, f"{name} is exported by the binding but not declared in the header"
    fake = _FakeLib()
    F._lib._declare(fake)
    typed = {n: f.argtypes for n, f in fake.fns.items() if f.argtypes is not None}
    assert len(typed) >= 30
    for name, args in typed.items():
        assert name in hdr, name
        assert len(args) == hdr[name], f"{name}: binding has {len(args)} parameters, header {hdr[name]}"


def test_physical_stack_arguments():
    """Argument handling of physical_to_spectral (no GPU): component tuples are stacked last, a
    single array is one field, complex input and mismatched grids are rejected."""
    import numpy as np
    import pytest
    from fit_gb300.api import _physical_stack
    assert _physical_stack((np.zeros((4, 6)), np.ones((4, 6)))).shape == (4, 6, 2)
    assert _physical_stack(np.zeros((4, 4, 4))).shape == (4, 4, 4, 1)
    with pytest.raises(ValueError):
        _physical_stack((np.zeros((4, 4)), np.zeros((4, 5))))
    with pytest.raises(ValueError):
        _physical_stack(np.zeros((4, 4), dtype=np.complex128))
    with pytest.raises(ValueError):
        _physical_stack(np.zeros((2, 2, 2, 2)))
    with pytest.raises(ValueError):
        _physical_stack(())


def test_direct_sum_rejects_three_halves():
    """DirectSumBackend with the exact 3/2 rule is an ArgumentError-class error, as in the reference
    (src/NonlinearTerm.jl:106-109, test/runtests.jl:341-343); raised before any device work."""
    import numpy as np
    import pytest
    ks = F.wavenumber_grid((8, 8), (2 * np.pi, 2 * np.pi))
    u = np.zeros((8, 8, 2), dtype=np.complex128)
    with pytest.raises(ValueError, match="PaddedThreeHalves"):
        F.compute_nonlinear_term(u, ks, dealiasing=F.PaddedThreeHalves(), spectral=F.DirectSumBackend())
    with pytest.raises(ValueError, match="PaddedThreeHalves"):
        F.calculate_spectral_flux(u, ks, dealiasing=F.PaddedThreeHalves(), spectral=F.DirectSumBackend())
