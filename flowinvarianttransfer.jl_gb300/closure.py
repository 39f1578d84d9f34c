"""Coarse-graining flux, the forced Navier-Stokes evolver and the learned subfilter-stress closure.

* ``calculate_coarse_graining_flux`` mirrors ``src/CoarseGrainingFlux.jl:60-72`` (physical velocity
  fields + coordinate vectors in, ``CoarseGrainingFluxResult`` out), in 2D and 3D, computed on the
  GPU with spectral filters (``src/Filters.jl:19-26``). The reference delegates the computation to
  the 2D-only CoarseGrainingEnergyFluxes.jl, which is not part of it.
* ``evolve_forced_navier_stokes`` advances ``û`` by SSP-RK3 steps of forced incompressible
  Navier-Stokes built on this library's nonlinear term.
* ``closure_data`` produces the closure's training/evaluation set on the device: the filtered
  velocity-gradient tensor ``A_ij = d_j ū_i`` (9 features), the exact subfilter stress ``tau``
  (6 targets) and the exact flux ``Pi_ell``.
* ``SubfilterStressMLP`` is the learned closure: a pointwise 9 -> 64 -> 64 -> 6 network trained and
  evaluated with the library's BF16 tensor-core kernels (FP32 accumulation). The exact
  coarse-graining path stays its fallback and the reference for its error.

Device data is held in torch tensors (allocation and streams only); every computation is a call
into libfit_gb300.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check
from .plan import get_plan
from .shells import wavenumber_grid
from .types import (AbstractFilter, CoarseGrainingFluxResult, CoarseGrainingFluxResultWithDiagnostics,
                    GaussianFilter, HelmholtzDecomposition, NoDecomposition, OrszagTwoThirds)


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise _lib.FitError("the closure path needs a CUDA device")
    return torch


def _stream():
    return _torch().cuda.current_stream().cuda_stream


def _vp(t):
    return None if t is None else C.c_void_p(t.data_ptr())


# ---- coarse-graining flux ------------------------------------------------------------------------

def _grid_lengths(coords_vecs):
    Ls = []
    for x in coords_vecs:
        x = np.asarray(x, dtype=np.float64)
        n = len(x)
        dx = (x[-1] - x[0]) / (n - 1) if n > 1 else 1.0
        Ls.append(n * dx)
    return Ls


def _strain_tensor(A, nd):
    S = np.empty(A.shape[:nd] + (nd, nd), dtype=A.dtype)
    for i in range(nd):
        for j in range(nd):
            S[..., i, j] = 0.5 * (A[..., i * nd + j] + A[..., j * nd + i])
    return S


def _stress_tensor(tau, nd):
    T = np.empty(tau.shape[:nd] + (nd, nd), dtype=tau.dtype)
    q = 0
    for i in range(nd):
        T[..., i, i] = tau[..., q]
        q += 1
    for i in range(nd):
        for j in range(i + 1, nd):
            T[..., i, j] = T[..., j, i] = tau[..., q]
            q += 1
    return T


def calculate_coarse_graining_flux(velocity_fields, coords_vecs, ell, filter=GaussianFilter(),
                                   decomposition=NoDecomposition(), return_diagnostics=False, precision=64):
    """Pointwise cross-scale flux ``Pi_ell(x) = -tau_ij S_ij`` (``src/CoarseGrainingFlux.jl:60-72``).

    ``velocity_fields``: tuple of D real arrays (shape ``ns``); ``coords_vecs``: tuple of nd uniform
    periodic coordinate vectors. ``decomposition``: ``NoDecomposition`` or, in 2D,
    ``HelmholtzDecomposition`` (a dict ``{"rotational": r, "divergent": d}`` of results, the exact
    periodic split). Returns ``CoarseGrainingFluxResult`` or, with ``return_diagnostics``,
    ``CoarseGrainingFluxResultWithDiagnostics`` (``tau`` and ``strain`` of shape ``ns + (nd, nd)``)."""
    if not isinstance(filter, AbstractFilter):
        raise TypeError("filter must be SharpSpectralFilter(), GaussianFilter() or TopHatFilter()")
    fields = tuple(np.asarray(f) for f in velocity_fields)
    nd = len(coords_vecs)
    if len(fields) != nd:
        raise ValueError(f"Number of velocity components ({len(fields)}) must equal number of spatial "
                         f"dimensions ({nd})")
    if nd not in (2, 3):
        raise ValueError("coarse-graining flux is defined here for 2D and 3D grids")
    ns = fields[0].shape
    if len(ns) != nd or any(f.shape != ns for f in fields):
        raise ValueError("velocity components must share the grid shape of the coordinates")
    ks = wavenumber_grid(ns, _grid_lengths(coords_vecs))
    plan = get_plan(ns, nd, nd, "none", precision, True, ks)
    u_hat = plan.forward_spectrum(np.stack(fields, axis=-1))

    def one(uh):
        Pi, mean, A, tau = plan.coarse_graining_flux(uh, ell, filter.code, diagnostics=return_diagnostics)
        if return_diagnostics:
            return CoarseGrainingFluxResultWithDiagnostics(float(ell), np.asarray(Pi), mean,
                                                           _stress_tensor(tau, nd), _strain_tensor(A, nd))
        return CoarseGrainingFluxResult(float(ell), np.asarray(Pi), mean)

    if isinstance(decomposition, NoDecomposition):
        return one(u_hat)
    if isinstance(decomposition, HelmholtzDecomposition) and nd == 2:
        rot, div = plan.helmholtz(u_hat)
        return {"rotational": one(rot), "divergent": one(div)}
    raise ValueError(f"{type(decomposition).__name__} is not available for the coarse-graining flux "
                     "(2D HelmholtzDecomposition or NoDecomposition)")


# ---- forced Navier-Stokes ------------------------------------------------------------------------

def evolve_forced_navier_stokes(u_hat, ks, nsteps, dt, nu, kf=2.0, power=0.1, dealiasing=OrszagTwoThirds(),
                                precision=64):
    """``nsteps`` SSP-RK3 steps of ``dû/dt = -P[N(û)] - nu k^2 û + alpha û 1[0<|k|<=kf]`` with
    ``alpha = power / (2 E_f)`` (constant power injection), ``û = fft(u)/Np``. Returns the new ``û``."""
    nd = len(ks)
    ns = tuple(np.asarray(u_hat).shape[:nd])
    f64 = np.asarray(u_hat).dtype != np.complex64
    plan = get_plan(ns, nd, nd, dealiasing.key, precision, f64, ks)
    return plan.ns_evolve(u_hat, nsteps, dt, nu, kf, power)


def evolve_forced_navier_stokes_device(u_hat_dev, ks, nsteps, dt, nu, kf=2.0, power=0.1, precision=32):
    """In-place device variant: ``u_hat_dev`` is a torch complex tensor of shape ``(nd, *reversed(ns))``
    (component slowest, x fastest: the column-major ``(ns..., nd)`` layout)."""
    torch = _torch()
    nd = len(ks)
    ns = tuple(int(n) for n in reversed(u_hat_dev.shape[1:]))
    if u_hat_dev.shape[0] != nd or not u_hat_dev.is_contiguous():
        raise ValueError("u_hat_dev must be a contiguous (nd, ...) complex tensor")
    f64 = u_hat_dev.dtype == torch.complex128
    plan = get_plan(ns, nd, nd, "two_thirds", precision, f64, ks)
    plan.set_stream(_stream())
    plan.ns_evolve_device(u_hat_dev.data_ptr(), nsteps, dt, nu, kf, power)


# ---- closure data --------------------------------------------------------------------------------

@dataclass
class ClosureData:
    """Field-major device tensors over n points (x fastest): A (9, n), tau (6, n), Pi (n)."""
    A: object
    tau: object
    Pi: object
    ell: float
    n: int
    mean_flux: float


def closure_data(u_hat_dev, ks, ell, filter=GaussianFilter()):
    """Exact coarse-graining quantities of a 3D complex64 device field ``(3, N2, N1, N0)``."""
    torch = _torch()
    ns = tuple(int(n) for n in reversed(u_hat_dev.shape[1:]))
    if len(ns) != 3 or u_hat_dev.shape[0] != 3 or u_hat_dev.dtype != torch.complex64:
        raise ValueError("closure_data takes a contiguous complex64 (3, N, N, N) device tensor")
    n = int(np.prod(ns))
    plan = get_plan(ns, 3, 3, "none", 32, False, ks)
    plan.set_stream(_stream())
    dev = u_hat_dev.device
    A = torch.empty((9, n), dtype=torch.float32, device=dev)
    tau = torch.empty((6, n), dtype=torch.float32, device=dev)
    Pi = torch.empty((n,), dtype=torch.float32, device=dev)
    mean = plan.coarse_graining_flux_device(u_hat_dev.data_ptr(), ell, filter.code, Pi.data_ptr(), A.data_ptr(),
                                            tau.data_ptr())
    return ClosureData(A, tau, Pi, float(ell), n, mean)


def field_compare(a, b):
    """(correlation, relative L2 error |a - b| / |b|) of two float32 device vectors."""
    torch = _torch()
    out = torch.empty(6, dtype=torch.float64, device=a.device)
    n = a.numel()
    check(_lib.load().fit_field_compare(_vp(a), _vp(b), n, _vp(out), _stream()))
    sa, sb, saa, sbb, sab, sdd = out.tolist()
    va = saa - sa * sa / n
    vb = sbb - sb * sb / n
    corr = (sab - sa * sb / n) / math.sqrt(va * vb) if va > 0 and vb > 0 else 0.0
    rel = math.sqrt(sdd / sbb) if sbb > 0 else float("inf")
    return corr, rel


def gradient_model_flux(data: ClosureData, p0=0, p1=None):
    """Pi of the gradient (Clark) model on points [p0, p1)."""
    torch = _torch()
    p1 = data.n if p1 is None else p1
    Pi = torch.empty(p1 - p0, dtype=torch.float32, device=data.A.device)
    X = data.A[:, p0:]
    check(_lib.load().fit_gradient_model_flux(_vp(X), data.n, p1 - p0, data.ell, None, _vp(Pi), _stream()))
    return Pi


# ---- the learned closure -------------------------------------------------------------------------

def init_params(seed=0):
    """He-uniform FP32 parameters in the kernel layout; padding (inputs 9..15, outputs 6..7) zero."""
    rng = np.random.default_rng(seed)
    W1 = np.zeros((64, 16))
    W1[:, :9] = rng.uniform(-1, 1, (64, 9)) * math.sqrt(6.0 / 9)
    W2 = rng.uniform(-1, 1, (64, 64)) * math.sqrt(6.0 / 64)
    W3 = np.zeros((8, 64))
    W3[:6] = rng.uniform(-1, 1, (6, 64)) * math.sqrt(3.0 / 64)
    return np.concatenate([W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), W3.ravel(),
                           np.zeros(8)]).astype(np.float32)


class SubfilterStressMLP:
    """A_ij (9) -> 64 -> 64 -> tau (6), ReLU; BF16 tensor-core kernels with FP32 accumulation.

    ``homogeneous`` (default): the network sees the direction v/|v| of the scaled gradient tensor
    and its output is multiplied by s = |v|^2, so the predicted stress is homogeneous of degree 2
    in A, as the exact subfilter stress is at leading order in ell.
    ``mixed``: the network learns the residual over the gradient (Clark) model, whose stress
    ell^2/12 A A^T is added in the forward kernel's epilogue (the filter scale is the training
    data's)."""

    def __init__(self, seed=0, device=None, params=None, homogeneous=True, mixed=False):
        torch = _torch()
        self.lib = _lib.load()
        self.nparam = int(self.lib.fit_mlp_nparams())
        dev = torch.device("cuda") if device is None else torch.device(device)
        p = init_params(seed) if params is None else np.asarray(params, dtype=np.float32)
        if p.size != self.nparam:
            raise ValueError(f"expected {self.nparam} parameters")
        self.params = torch.from_numpy(p.copy()).to(dev)
        self.grad = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.loss = torch.zeros(1, dtype=torch.float64, device=dev)
        self.in_scale = torch.ones(9, dtype=torch.float32, device=dev)
        self.t_scale = torch.ones(6, dtype=torch.float32, device=dev)
        self.step = 0
        self.device = dev
        self.homogeneous = bool(homogeneous)
        self.mixed = bool(mixed)
        self.ell = 0.0

    # scales: unit variance of every feature and target over the training points
    def fit_scales(self, X, T, ld, P):
        torch = _torch()
        mx = torch.empty(18, dtype=torch.float64, device=self.device)
        mt = torch.empty(12, dtype=torch.float64, device=self.device)
        check(self.lib.fit_field_moments(_vp(X), ld, P, 9, _vp(mx), _stream()))
        check(self.lib.fit_field_moments(_vp(T), ld, P, 6, _vp(mt), _stream()))
        mx = mx.view(9, 2)
        mt = mt.view(6, 2)
        sx = (mx[:, 1] / P - (mx[:, 0] / P) ** 2).clamp_min(1e-30).sqrt()
        st = (mt[:, 1] / P).clamp_min(1e-30).sqrt()   # targets are not centred: the bias learns the mean
        self.in_scale.copy_((1.0 / sx).float())
        # homogeneous form: outputs are multiplied by s = |v|^2, whose mean is sum_f E[x_f^2] / var_f
        gain = float((mx[:, 1] / P / sx ** 2).sum()) if self.homogeneous else 1.0
        self.t_scale.copy_((gain / st).float())

    def grad_of(self, X, T, ld, P, Ptot=None):
        """Gradient of the scaled MSE over points [0, P) of field-major X/T (stride ld)."""
        self.grad.zero_()
        self.loss.zero_()
        check(self.lib.fit_mlp_train_grad(_vp(self.params), _vp(X), _vp(T), ld, P, P if Ptot is None else Ptot,
                                          _vp(self.in_scale), _vp(self.t_scale), int(self.homogeneous),
                                          _vp(self.grad), _vp(self.loss), _stream()))
        return self.grad, self.loss

    def train(self, data: ClosureData, p0, p1, steps=1500, batch=65536, lr=2e-3, seed=0, log_every=0):
        """Adam on random contiguous slabs of ``batch`` points from [p0, p1); cosine learning-rate decay.
        Returns the list of (step, mean scaled loss) at ``log_every``."""
        rng = np.random.default_rng(seed)
        self.ell = float(data.ell)
        X, T, ld = data.A, self.targets(data), data.n
        self.fit_scales(X[:, p0:], T[:, p0:], ld, p1 - p0)
        hist = []
        for s in range(steps):
            off = p0 + int(rng.integers(0, max(1, p1 - p0 - batch + 1)))
            P = min(batch, p1 - off)
            self.grad_of(X[:, off:], T[:, off:], ld, P)
            self.step += 1
            lr_s = lr * 0.5 * (1.0 + math.cos(math.pi * s / steps))
            check(self.lib.fit_mlp_adam(_vp(self.params), _vp(self.grad), _vp(self.m), _vp(self.v), self.step,
                                        C.c_float(lr_s), C.c_float(0.9), C.c_float(0.999), C.c_float(1e-8),
                                        _stream()))
            if log_every and (s % log_every == 0 or s == steps - 1):
                hist.append((s, float(self.loss.item()) / (6 * P)))
        return hist

    def targets(self, data: ClosureData):
        """The training targets: the exact stress, or its residual over the gradient model."""
        if not self.mixed:
            return data.tau
        torch = _torch()
        R = getattr(data, "residual", None)
        if R is None or getattr(data, "residual_ell", None) != data.ell:
            R = torch.empty_like(data.tau)
            check(self.lib.fit_stress_residual(_vp(data.A), _vp(data.tau), data.n, data.n, data.ell, _vp(R),
                                               _stream()))
            data.residual, data.residual_ell = R, data.ell
        return R

    def predict(self, X, ld, P, want_tau=True, want_flux=True):
        """Predicted stress (6, P) and/or flux (P) for points [0, P) of X (stride ld)."""
        torch = _torch()
        Y = torch.empty((6, ld), dtype=torch.float32, device=self.device) if want_tau else None
        Pi = torch.empty(P, dtype=torch.float32, device=self.device) if want_flux else None
        check(self.lib.fit_mlp_forward(_vp(self.params), _vp(X), ld, P, _vp(self.in_scale), _vp(self.t_scale),
                                       int(self.homogeneous), self.ell if self.mixed else 0.0, _vp(Y), _vp(Pi),
                                       _stream()))
        return (Y[:, :P] if Y is not None else None), Pi

    def evaluate(self, data: ClosureData, p0, p1):
        """Pi_ell correlation and relative L2 error on points [p0, p1) for the MLP, the gradient
        model and no closure (Pi = 0), against the exact coarse-graining flux."""
        P = p1 - p0
        X = data.A[:, p0:]
        _, Pi_mlp = self.predict(X, data.n, P, want_tau=False)
        exact = data.Pi[p0:p1]
        c_mlp, r_mlp = field_compare(Pi_mlp, exact)
        Pi_grad = gradient_model_flux(data, p0, p1)
        c_grad, r_grad = field_compare(Pi_grad, exact)
        return {"corr_mlp": c_mlp, "rel_l2_mlp": r_mlp, "corr_gradient_model": c_grad,
                "rel_l2_gradient_model": r_grad, "corr_no_closure": 0.0, "rel_l2_no_closure": 1.0,
                "points": P}
