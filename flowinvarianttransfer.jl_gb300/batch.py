"""Uneven batches: many spectral-flux instances (2D and 3D grids of different sizes, kinetic-energy
and passive-scalar invariants, isotropic / perpendicular / parallel shells) computed as one CUDA
graph launch, with the transform kernels chosen by the library's autotuner.

Each instance is what ``calculate_spectral_flux`` / ``calculate_scalar_flux``
(``src/SpectralFlux.jl:49-122,203-215``) computes for it; the reference evaluates such a set one
call at a time. Device buffers are torch tensors (allocation only); all arithmetic runs in
libfit_gb300.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check
from .api import _as_component_field, _shells
from .plan import Plan, _dptr
from .types import IsotropicShells, KineticEnergy, OrszagTwoThirds, PassiveScalar, SpectralFluxResult


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise _lib.FitError("batched flux needs a CUDA device")
    return torch


def _to_device(a, cdtype):
    """(ns..., M) array -> flat device tensor holding its column-major data."""
    torch = _torch()
    raw = np.asfortranarray(np.asarray(a).astype(cdtype, copy=False)).ravel(order="F")
    return torch.from_numpy(raw.copy()).cuda()


class SpectralFluxBatch:
    """A fixed set of flux instances run as one graph launch.

    ``instances``: dicts with ``velocity_hat`` ``(ns..., D)`` and ``ks``, and optionally
    ``scalar_hat`` (passive-scalar flux advected by the velocity), ``binning``, ``geometry``
    (``IsotropicShells()``, ``PerpendicularShells()``, ``ParallelShells(dims)``), ``invariant`` and
    ``dealiasing``. ``precision`` 32 keeps fields in complex64 with FP32 transforms and FP64 shell
    sums; 64 is FP64 throughout. The first :meth:`run` executes eagerly (allocation, autotuning),
    the second captures and launches the graph, later runs launch it."""

    def __init__(self, instances, precision=32, n_branches=8, autotune=True):
        torch = _torch()
        self.lib = _lib.load()
        self.precision = int(precision)
        cdt = np.complex128 if self.precision == 64 else np.complex64
        check(self.lib.fit_autotune_enable(int(bool(autotune))))
        h = C.c_void_p()
        check(self.lib.fit_batch_create(C.byref(h), int(n_branches)))
        self.h = h
        self.items = []
        self.stream = torch.cuda.current_stream().cuda_stream
        for spec in instances:
            ks = spec["ks"]
            nd = len(ks)
            if "ns" in spec:
                # device-resident inputs: flat tensors holding column-major (ns..., comp) data
                ns = tuple(int(n) for n in spec["ns"])
                vdev, sdev = spec["velocity_dev"], spec.get("scalar_dev")
            else:
                v = _as_component_field(spec["velocity_hat"], nd)
                ns = v.shape[:nd]
                vdev = _to_device(v, cdt)
                s = spec.get("scalar_hat")
                sdev = _to_device(_as_component_field(s, nd), cdt) if s is not None else None
            self._add(spec, ks, ns, vdev, sdev, cdt)

    def _add(self, spec, ks, ns, vdev, sdev, cdt):
        torch = _torch()
        want = torch.complex128 if cdt == np.complex128 else torch.complex64
        for t in (vdev, sdev):
            if t is not None and (t.dtype != want or not t.is_cuda or not t.is_contiguous()):
                raise ValueError(f"device inputs must be contiguous {want} CUDA tensors")
        Ntot = int(np.prod(ns))
        D = vdev.numel() // Ntot
        if sdev is not None:
            fd, ad, inv, M = sdev, vdev, PassiveScalar(), sdev.numel() // Ntot
        else:
            fd, ad, inv, M = vdev, None, spec.get("invariant", KineticEnergy()), D
        geometry = spec.get("geometry", IsotropicShells())
        binning, edges, centers, dm, f32 = _shells(ks, spec.get("binning"), geometry)
        dealias = spec.get("dealiasing", OrszagTwoThirds())
        plan = Plan(ns, M, D, dealias.key, self.precision, self.precision == 64, ks)
        plan.set_stream(self.stream)
        nsh = len(edges) - 1
        T = torch.zeros(nsh, dtype=torch.float64, device="cuda")
        Pi = torch.zeros(nsh, dtype=torch.float64, device="cuda")
        check(self.lib.fit_batch_add_flux(self.h, plan.h, C.c_void_p(fd.data_ptr()),
                                          C.c_void_p(ad.data_ptr()) if ad is not None else None, _dptr(edges),
                                          len(edges), dm, int(f32), inv.code, C.c_void_p(T.data_ptr()),
                                          C.c_void_p(Pi.data_ptr())))
        ft = np.float32 if self.precision == 32 else np.float64
        self.items.append({"plan": plan, "f": fd, "a": ad, "T": T, "Pi": Pi, "centers": centers.astype(ft),
                           "ft": ft, "edges": edges, "ns": ns, "invariant": inv, "geometry": geometry})

    def run(self):
        """One batch execution, asynchronous on the stream current at construction."""
        check(self.lib.fit_batch_run(self.h, C.c_void_p(self.stream)))

    def run_eager(self):
        """Every instance launched one after the other on the stream, without the graph."""
        check(self.lib.fit_batch_run_eager(self.h, C.c_void_p(self.stream)))

    def results(self):
        """SpectralFluxResult per instance (synchronises)."""
        torch = _torch()
        torch.cuda.synchronize()
        out = []
        for it in self.items:
            ft = it["ft"]
            T = it["T"].cpu().numpy()
            out.append(SpectralFluxResult(it["centers"], T.astype(ft), it["Pi"].cpu().numpy().astype(ft)))
        return out

    def info(self):
        v = (C.c_int64 * 4)()
        check(self.lib.fit_batch_info(self.h, v, 4))
        return {"instances": v[0], "state": v[1], "graph_kernels": v[2], "branches": v[3]}

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fit_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def calculate_spectral_flux_batch(instances, precision=32, n_branches=8, autotune=True):
    """Spectral flux of every instance (see :class:`SpectralFluxBatch`), one graph launch for all."""
    b = SpectralFluxBatch(instances, precision=precision, n_branches=n_branches, autotune=autotune)
    b.run()
    b.run()   # graph capture + launch
    res = b.results()
    b.close()
    return res


def autotune_summary():
    """Autotuner table: summary and one dict per tuned pass shape."""
    lib = _lib.load()
    n, c = C.c_int64(), C.c_int64()
    md, mb = C.c_double(), C.c_double()
    check(lib.fit_autotune_info(C.byref(n), C.byref(c), C.byref(md), C.byref(mb)))
    kinds = ("strided_fwd", "strided_inv", "c2r_x", "r2c_x")
    entries = []
    for i in range(n.value):
        f = (C.c_int64 * 9)()
        ms = (C.c_double * 2)()
        check(lib.fit_autotune_entry(i, f, ms))
        entries.append({"kind": kinds[f[0]], "N": f[1], "cols": f[2], "batch": f[3], "elem_bytes": f[4],
                        "engine": "compile-time" if f[5] == 0 else "runtime", "C": f[6], "ept": f[7],
                        "radix_order": ("8s first", "4s first", "8s last")[f[8]] if f[5] else None,
                        "ms_best": ms[0], "ms_default": ms[1]})
    return {"entries": n.value, "runtime_engine_chosen": c.value, "ms_default_sum": md.value,
            "ms_best_sum": mb.value, "table": entries}


def autotune_enable(on=True):
    check(_lib.load().fit_autotune_enable(int(bool(on))))


def autotune_clear():
    check(_lib.load().fit_autotune_clear())
