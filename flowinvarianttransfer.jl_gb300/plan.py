"""``Plan``: one libfit_gb300 plan (device workspace, transform tables, stream) for a grid.

This is the host-side counterpart of the reference's workspace + plan bundle
(``src/Workspaces.jl:46-75``, ``ext/FlowInvariantTransferFFTWExt.jl:26-49``): it owns the device
buffers and the C handle and frees them when collected. Array arguments are numpy arrays in the
reference layout (``(ns..., comp)``, any memory order; copied to column-major) or, for the
``*_device`` calls, raw device pointers to column-major data.
"""
from __future__ import annotations

import ctypes as C
import threading
from collections import OrderedDict

import numpy as np

from . import _lib
from ._lib import PTR_DEVICE, PTR_HOST, check


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Plan:
    def __init__(self, ns, n_advected, n_advecting, dealias, precision, io_f64, ks):
        lib = _lib.load()
        self.lib = lib
        self.ns = tuple(int(n) for n in ns)
        self.nd = len(self.ns)
        self.M = int(n_advected)
        self.D = int(n_advecting)
        self.dealias = dealias
        self.precision = int(precision)
        self.io_f64 = bool(io_f64)
        self.cdtype = np.complex128 if self.io_f64 else np.complex64
        self._ks = [np.ascontiguousarray(np.asarray(k, dtype=np.float64)) for k in ks]
        arr = (C.POINTER(C.c_double) * self.nd)(*[_dptr(k) for k in self._ks])
        nsv = (C.c_int64 * self.nd)(*self.ns)
        h = C.c_void_p()
        check(lib.fit_plan_create(C.byref(h), self.nd, nsv, self.M, self.D, _lib.DEALIAS[dealias],
                                  self.precision, int(self.io_f64), arr))
        self.h = h
        self.lock = threading.Lock()

    def __del__(self):
        try:
            if getattr(self, "h", None) and self.h.value:
                self.lib.fit_plan_destroy(self.h)
                self.h = C.c_void_p()
        except Exception:
            pass

    # ---- helpers ----
    def _field(self, a, ncomp):
        a = np.asarray(a)
        if a.ndim == self.nd:
            a = a[..., None]
        if a.shape != self.ns + (ncomp,):
            raise ValueError(f"field has shape {a.shape}; expected {self.ns + (ncomp,)}")
        return np.asfortranarray(a.astype(self.cdtype, copy=False))

    @staticmethod
    def _vp(a):
        return None if a is None else C.c_void_p(a.ctypes.data)

    def info(self):
        out = (C.c_int64 * 9)()
        check(self.lib.fit_plan_info(self.h, out, 9))
        return list(out)

    def set_stream(self, stream_ptr: int):
        check(self.lib.fit_plan_set_stream(self.h, C.c_void_p(stream_ptr)))

    # ---- host-array entry points ----
    def nonlinear_term(self, f_hat, adv_hat=None):
        f = self._field(f_hat, self.M)
        a = None if adv_hat is None else self._field(adv_hat, self.D)
        out = np.empty(self.ns + (self.M,), dtype=self.cdtype, order="F")
        with self.lock:
            check(self.lib.fit_nonlinear_term(self.h, self._vp(f), self._vp(a), self._vp(out), PTR_HOST))
        return out

    def assign_shells(self, edges, dmask, coord_f32):
        e = np.ascontiguousarray(edges, dtype=np.float64)
        out = np.empty(self.ns, dtype=np.int64, order="F")
        with self.lock:
            check(self.lib.fit_assign_shells(self.h, _dptr(e), len(e), dmask, int(coord_f32), self._vp(out), PTR_HOST))
        return out

    def transfer_density(self, inv, carrier, nhat):
        c = self._field(carrier, self.M)
        n = self._field(nhat, self.M)
        out = np.empty(self.ns, dtype=np.float64, order="F")
        with self.lock:
            check(self.lib.fit_transfer_density(self.h, inv, self._vp(c), self._vp(n), self._vp(out), PTR_HOST))
        return out

    def spectral_flux(self, u_hat, edges, dmask, coord_f32, inv, adv_hat=None, carrier=None):
        u = self._field(u_hat, self.M)
        a = None if adv_hat is None else self._field(adv_hat, self.D)
        c = None if carrier is None else self._field(carrier, self.M)
        e = np.ascontiguousarray(edges, dtype=np.float64)
        T = np.zeros(len(e) - 1)
        P = np.zeros(len(e) - 1)
        with self.lock:
            check(self.lib.fit_spectral_flux(self.h, self._vp(u), self._vp(a), self._vp(c), _dptr(e), len(e), dmask,
                                             int(coord_f32), inv, self._vp(T), self._vp(P), PTR_HOST))
        return T, P

    def shell_to_shell(self, u_hat, edges, dmask, coord_f32, inv, mode, verify=True, adv_hat=None):
        u = self._field(u_hat, self.M)
        a = None if adv_hat is None else self._field(adv_hat, self.D)
        e = np.ascontiguousarray(edges, dtype=np.float64)
        n = len(e) - 1
        T = np.zeros((n, n), order="F")
        net = np.zeros(n)
        asym = np.zeros(1)
        with self.lock:
            check(self.lib.fit_shell_to_shell(self.h, self._vp(u), self._vp(a), _dptr(e), len(e), dmask,
                                              int(coord_f32), inv, mode, int(verify), self._vp(T), self._vp(net),
                                              self._vp(asym), PTR_HOST))
        return T, net, float(asym[0])

    def set_shell_index(self, shell_idx, n_shells):
        """Install a precomputed shell index (Int64, 1-based, 0 = none; the ``ws.shell_idx`` of the
        reference's ShellToShellWorkspace) as this plan's shell table."""
        idx = np.asarray(shell_idx)
        if idx.shape != self.ns:
            raise ValueError(f"shell index has shape {idx.shape}; expected {self.ns}")
        idx = np.asfortranarray(idx.astype(np.int64, copy=False))
        with self.lock:
            check(self.lib.fit_set_shell_index(self.h, self._vp(idx), int(n_shells), PTR_HOST))

    def shell_to_shell_indexed(self, u_hat, n_shells, inv, mode, verify=True, adv_hat=None):
        """shell_to_shell binned by the index installed with set_shell_index."""
        u = self._field(u_hat, self.M)
        a = None if adv_hat is None else self._field(adv_hat, self.D)
        n = int(n_shells)
        T = np.zeros((n, n), order="F")
        net = np.zeros(n)
        asym = np.zeros(1)
        with self.lock:
            check(self.lib.fit_shell_to_shell_indexed(self.h, self._vp(u), self._vp(a), inv, mode, int(verify),
                                                      self._vp(T), self._vp(net), self._vp(asym), PTR_HOST))
        return T, net, float(asym[0])

    def band_to_band(self, u_hat, centers, logwidth, dmask, coord_f32, inv, adv_hat=None):
        u = self._field(u_hat, self.M)
        a = None if adv_hat is None else self._field(adv_hat, self.D)
        c = np.ascontiguousarray(centers, dtype=np.float64)
        nb = len(c)
        T = np.zeros((nb, nb), order="F")
        net = np.zeros(nb)
        asym = np.zeros(1)
        with self.lock:
            check(self.lib.fit_band_to_band(self.h, self._vp(u), self._vp(a), _dptr(c), nb, float(logwidth), dmask,
                                            int(coord_f32), inv, self._vp(T), self._vp(net), self._vp(asym),
                                            PTR_HOST))
        return T, net, float(asym[0])

    def helical(self, u_hat):
        u = self._field(u_hat, self.M)
        up = np.empty(self.ns + (3,), dtype=self.cdtype, order="F")
        um = np.empty_like(up)
        with self.lock:
            check(self.lib.fit_helical_decompose(self.h, self._vp(u), self._vp(up), self._vp(um), PTR_HOST))
        return up, um

    def toroidal_poloidal(self, u_hat):
        u = self._field(u_hat, self.M)
        t = np.empty(self.ns + (3,), dtype=self.cdtype, order="F")
        q = np.empty_like(t)
        with self.lock:
            check(self.lib.fit_toroidal_poloidal_decompose(self.h, self._vp(u), self._vp(t), self._vp(q), PTR_HOST))
        return t, q

    def helmholtz(self, u_hat):
        u = self._field(u_hat, self.M)
        r = np.empty(self.ns + (2,), dtype=self.cdtype, order="F")
        d = np.empty_like(r)
        with self.lock:
            check(self.lib.fit_helmholtz_decompose(self.h, self._vp(u), self._vp(r), self._vp(d), PTR_HOST))
        return r, d

    def partial_fluxes(self, u_hat, decomposition, inv, edges, dmask, coord_f32):
        u = self._field(u_hat, self.M)
        e = np.ascontiguousarray(edges, dtype=np.float64)
        n = len(e) - 1
        out = np.zeros(8 * n)
        with self.lock:
            check(self.lib.fit_partial_fluxes(self.h, self._vp(u), decomposition, inv, _dptr(e), len(e), dmask,
                                              int(coord_f32), self._vp(out), PTR_HOST))
        return out.reshape(8, n)

    def partial_fluxes_batched(self, u_hat, decomposition, invs, edges, dmask, coord_f32):
        u = self._field(u_hat, self.M)
        e = np.ascontiguousarray(edges, dtype=np.float64)
        n = len(e) - 1
        iv = (C.c_int * len(invs))(*invs)
        out = np.zeros(len(invs) * 8 * n)
        with self.lock:
            check(self.lib.fit_partial_fluxes_batched(self.h, self._vp(u), decomposition, iv, len(invs), _dptr(e),
                                                      len(e), dmask, int(coord_f32), self._vp(out), PTR_HOST))
        return out.reshape(len(invs), 8, n)

    def spectral_flux_device(self, u_ptr, a_ptr, c_ptr, edges, dmask, coord_f32, inv, T_ptr, P_ptr):
        e = np.ascontiguousarray(edges, dtype=np.float64)
        check(self.lib.fit_spectral_flux(self.h, C.c_void_p(u_ptr), C.c_void_p(a_ptr) if a_ptr else None,
                                         C.c_void_p(c_ptr) if c_ptr else None, _dptr(e), len(e), dmask,
                                         int(coord_f32), inv, C.c_void_p(T_ptr), C.c_void_p(P_ptr), PTR_DEVICE))

    def partial_fluxes_device(self, u_ptr, decomposition, inv, edges, dmask, coord_f32, T_ptr):
        e = np.ascontiguousarray(edges, dtype=np.float64)
        check(self.lib.fit_partial_fluxes(self.h, C.c_void_p(u_ptr), decomposition, inv, _dptr(e), len(e), dmask,
                                          int(coord_f32), C.c_void_p(T_ptr), PTR_DEVICE))

    def partial_fluxes_batched_device(self, u_ptr, decomposition, invs, edges, dmask, coord_f32, T_ptr):
        e = np.ascontiguousarray(edges, dtype=np.float64)
        iv = (C.c_int * len(invs))(*invs)
        check(self.lib.fit_partial_fluxes_batched(self.h, C.c_void_p(u_ptr), decomposition, iv, len(invs), _dptr(e),
                                                  len(e), dmask, int(coord_f32), C.c_void_p(T_ptr), PTR_DEVICE))

    def mode_to_mode(self, u_hat, inv, fp64=True, adv_hat=None):
        u = self._field(u_hat, self.M)
        a = None if adv_hat is None else self._field(adv_hat, self.D)
        nm = int(np.prod(self.ns))
        S = np.empty(self.ns + self.ns, dtype=np.float64, order="F")
        net = np.empty(self.ns, dtype=np.float64, order="F")
        with self.lock:
            check(self.lib.fit_mode_to_mode(self.h, self._vp(u), self._vp(a), inv, int(fp64), self._vp(S),
                                            self._vp(net), PTR_HOST))
        return S, net

    def forward_spectrum(self, u_phys):
        """û = fft(u)/Np of real physical fields (ns..., M) computed on the device."""
        rdt = np.float64 if self.io_f64 else np.float32
        u = np.asarray(u_phys)
        if u.ndim == self.nd:
            u = u[..., None]
        if u.shape != self.ns + (self.M,):
            raise ValueError(f"field has shape {u.shape}; expected {self.ns + (self.M,)}")
        u = np.asfortranarray(u.astype(rdt, copy=False))
        out = np.empty(self.ns + (self.M,), dtype=self.cdtype, order="F")
        with self.lock:
            check(self.lib.fit_forward_spectrum(self.h, self._vp(u), self._vp(out), PTR_HOST))
        return out

    def coarse_graining_flux(self, u_hat, ell, filter_code, diagnostics=False):
        u = self._field(u_hat, self.M)
        rdt = np.float64 if self.precision == 64 else np.float32
        nd = self.nd
        Pi = np.empty(self.ns, dtype=rdt, order="F")
        A = np.empty(self.ns + (nd * nd,), dtype=rdt, order="F") if diagnostics else None
        tau = np.empty(self.ns + (nd * (nd + 1) // 2,), dtype=rdt, order="F") if diagnostics else None
        mean = C.c_double()
        with self.lock:
            check(self.lib.fit_coarse_graining_flux(self.h, self._vp(u), float(ell), int(filter_code), self._vp(Pi),
                                                    self._vp(A), self._vp(tau), C.byref(mean), PTR_HOST))
        return Pi, float(mean.value), A, tau

    def ns_evolve(self, u_hat, nsteps, dt, nu, kf, power):
        u = np.array(self._field(u_hat, self.M), order="F", copy=True)
        with self.lock:
            check(self.lib.fit_ns_evolve(self.h, self._vp(u), int(nsteps), float(dt), float(nu), float(kf),
                                         float(power), PTR_HOST))
        return u

    # ---- device-pointer entry points (inputs already resident in HBM) ----
    def shell_to_shell_device(self, u_ptr, a_ptr, edges, dmask, coord_f32, inv, mode, T_ptr, net_ptr, asym_ptr,
                              verify=True):
        e = np.ascontiguousarray(edges, dtype=np.float64)
        check(self.lib.fit_shell_to_shell(self.h, C.c_void_p(u_ptr), C.c_void_p(a_ptr) if a_ptr else None, _dptr(e),
                                          len(e), dmask, int(coord_f32), inv, mode, int(verify), C.c_void_p(T_ptr),
                                          C.c_void_p(net_ptr) if net_ptr else None,
                                          C.c_void_p(asym_ptr) if asym_ptr else None, PTR_DEVICE))


    def band_to_band_device(self, u_ptr, a_ptr, centers, logwidth, dmask, coord_f32, inv, T_ptr, net_ptr,
                            asym_ptr):
        c = np.ascontiguousarray(centers, dtype=np.float64)
        check(self.lib.fit_band_to_band(self.h, C.c_void_p(u_ptr), C.c_void_p(a_ptr) if a_ptr else None, _dptr(c),
                                        len(c), float(logwidth), dmask, int(coord_f32), inv, C.c_void_p(T_ptr),
                                        C.c_void_p(net_ptr) if net_ptr else None,
                                        C.c_void_p(asym_ptr) if asym_ptr else None, PTR_DEVICE))

    def mode_to_mode_device(self, u_ptr, inv, fp64, S_ptr, net_ptr):
        check(self.lib.fit_mode_to_mode(self.h, C.c_void_p(u_ptr), None, inv, int(fp64), C.c_void_p(S_ptr),
                                        C.c_void_p(net_ptr), PTR_DEVICE))

    def coarse_graining_flux_device(self, u_ptr, ell, filter_code, Pi_ptr, A_ptr=0, tau_ptr=0):
        mean = C.c_double()
        check(self.lib.fit_coarse_graining_flux(self.h, C.c_void_p(u_ptr), float(ell), int(filter_code),
                                                C.c_void_p(Pi_ptr), C.c_void_p(A_ptr) if A_ptr else None,
                                                C.c_void_p(tau_ptr) if tau_ptr else None, C.byref(mean),
                                                PTR_DEVICE))
        return float(mean.value)

    def ns_evolve_device(self, u_ptr, nsteps, dt, nu, kf, power):
        check(self.lib.fit_ns_evolve(self.h, C.c_void_p(u_ptr), int(nsteps), float(dt), float(nu), float(kf),
                                     float(power), PTR_DEVICE))

    def forward_spectrum_device(self, u_ptr, out_ptr):
        check(self.lib.fit_forward_spectrum(self.h, C.c_void_p(u_ptr), C.c_void_p(out_ptr), PTR_DEVICE))


_CACHE: "OrderedDict[tuple, Plan]" = OrderedDict()
_CACHE_LOCK = threading.Lock()
_CACHE_MAX = 6


def get_plan(ns, M, D, dealias, precision, io_f64, ks) -> Plan:
    key = (tuple(ns), M, D, dealias, precision, bool(io_f64),
           tuple(np.asarray(k, dtype=np.float64).tobytes() for k in ks))
    with _CACHE_LOCK:
        p = _CACHE.get(key)
        if p is not None:
            _CACHE.move_to_end(key)
            return p
        p = Plan(ns, M, D, dealias, precision, io_f64, ks)
        _CACHE[key] = p
        while len(_CACHE) > _CACHE_MAX:
            _CACHE.popitem(last=False)
        return p


def clear_plans():
    with _CACHE_LOCK:
        _CACHE.clear()
