"""FP64 numpy restatement of the closure data path (TEST ORACLE ONLY).

* ``ns_rhs`` / ``ns_evolve``: forced incompressible Navier-Stokes on the spectral state in the
  package convention ``û = fft(u)/Np``, SSP-RK3 (Shu-Osher) with the nonlinear term of
  ``fit_oracle.nonlinear_term`` (``ext/FlowInvariantTransferFFTWExt.jl:61-121``) scaled by ``Np^2``
  (that term transforms ``ifft(û) = u/Np``), Leray projection, viscosity and constant-power forcing
  of the shells ``0 < |k| <= kf``. The reference's evolvers (``examples/flows.jl:28-89``) are
  unforced RK2 with an integrating factor; this forced RK3 form restates the GPU evolver's
  equations, so it is unpinned against the reference.
* ``mlp_*``: the pointwise closure network 9 -> 64 -> 64 -> 6 (ReLU) with its analytic gradient,
  in FP64, optionally rounding to BF16 exactly where the tensor-core kernels do (features,
  hidden activations, output and hidden gradients). It has no reference counterpart.
* ``clark_stress``: the gradient (Clark) model ``tau_ij ~ ell^2/12 * A_ik A_jk`` for a Gaussian filter.
"""
from __future__ import annotations

import numpy as np

from .fit_oracle import _kcomp, keep_mask, nonlinear_term

# ---------------------------------------------------------------------------------------------
# Forced Navier-Stokes
# ---------------------------------------------------------------------------------------------


def ns_rhs(u_hat, ks, nu, kf, power, dealiasing="two_thirds"):
    nd = len(ks)
    ns = u_hat.shape[:nd]
    Np = float(np.prod(ns))
    N = nonlinear_term(u_hat, ks, dealiasing) * Np ** 2
    kc = [_kcomp(ks, d, ns) for d in range(nd)]
    k2 = sum(k * k for k in kc)
    kn = sum(kc[d] * N[..., d] for d in range(nd))
    with np.errstate(invalid="ignore", divide="ignore"):
        proj = np.where(k2 > 0, kn / np.where(k2 > 0, k2, 1.0), 0.0)
    PN = np.stack([N[..., d] - kc[d] * proj for d in range(nd)], axis=-1)
    forced = (k2 > 0) & (k2 <= kf * kf)
    Ef = 0.5 * np.sum(np.abs(u_hat[forced]) ** 2)
    alpha = power / (2.0 * Ef) if Ef > 0 else 0.0
    fac = -nu * k2 + alpha * forced
    return -PN + fac[..., None] * u_hat


def _restrict(u, ks, dealiasing):
    nd = len(ks)
    ns = u.shape[:nd]
    kc = [_kcomp(ks, d, ns) for d in range(nd)]
    k2 = sum(k * k for k in kc)
    keep = keep_mask(ns) if dealiasing == "two_thirds" else np.ones(ns, dtype=bool)
    return u * (keep & (k2 > 0))[..., None]


def ns_evolve(u_hat, ks, nsteps, dt, nu, kf, power, dealiasing="two_thirds"):
    """``nsteps`` SSP-RK3 steps: u1 = u0 + dt L(u0); u2 = 3/4 u0 + 1/4 (u1 + dt L(u1));
    u3 = 1/3 u0 + 2/3 (u2 + dt L(u2)); each stage restricted to the retained, non-DC modes."""
    u = np.array(u_hat, dtype=np.complex128)

    def L(v):
        return ns_rhs(v, ks, nu, kf, power, dealiasing)

    for _ in range(nsteps):
        u1 = _restrict(u + dt * L(u), ks, dealiasing)
        u2 = _restrict(0.75 * u + 0.25 * (u1 + dt * L(u1)), ks, dealiasing)
        u = _restrict(u / 3.0 + 2.0 / 3.0 * (u2 + dt * L(u2)), ks, dealiasing)
    return u


# ---------------------------------------------------------------------------------------------
# Closure MLP
# ---------------------------------------------------------------------------------------------

OFF = {"W1": (0, (64, 16)), "b1": (1024, (64,)), "W2": (1088, (64, 64)), "b2": (5184, (64,)),
       "W3": (5248, (8, 64)), "b3": (5760, (8,))}
NPARAM = 5768


def mlp_unpack(p):
    return {k: np.asarray(p[o:o + int(np.prod(s))], dtype=np.float64).reshape(s) for k, (o, s) in OFF.items()}


def mlp_pack(d):
    p = np.zeros(NPARAM)
    for k, (o, s) in OFF.items():
        p[o:o + int(np.prod(s))] = np.asarray(d[k], dtype=np.float64).ravel()
    return p


def mlp_init(seed=0):
    """He-uniform weights; padding (input columns 9..15, output rows 6..7) zero."""
    rng = np.random.default_rng(seed)
    d = {}
    d["W1"] = np.zeros((64, 16))
    d["W1"][:, :9] = rng.uniform(-1, 1, (64, 9)) * np.sqrt(6.0 / 9)
    d["b1"] = np.zeros(64)
    d["W2"] = rng.uniform(-1, 1, (64, 64)) * np.sqrt(6.0 / 64)
    d["b2"] = np.zeros(64)
    d["W3"] = np.zeros((8, 64))
    d["W3"][:6] = rng.uniform(-1, 1, (6, 64)) * np.sqrt(3.0 / 64)
    d["b3"] = np.zeros(8)
    return mlp_pack(d).astype(np.float32)


def bf16(x):
    """Round to bfloat16 (round to nearest, ties to even), returned as float64."""
    x32 = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    b = x32.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def _f32(x):
    return np.asarray(x, dtype=np.float32).astype(np.float64)


def mlp_forward(params, X, in_scale, t_scale, emulate_bf16=False, homogeneous=False, clark_ell=0.0):
    """X: (9, P) features; returns (Y (6, P) in target units, cache). ``homogeneous``: the network
    sees v/|v| (v: scaled features) and its output is multiplied by s = |v|^2. ``clark_ell`` > 0:
    the gradient-model stress at that filter scale is added (the network is a residual)."""
    d = mlp_unpack(params)
    r = bf16 if emulate_bf16 else (lambda v: v)
    W1, W2, W3 = r(d["W1"]), r(d["W2"]), r(d["W3"])
    P = X.shape[1]
    x = np.zeros((P, 16))
    x[:, :9] = (_f32(np.asarray(X, np.float32) * np.asarray(in_scale, np.float32)[:, None]) if emulate_bf16
                else np.asarray(X, np.float64) * np.asarray(in_scale, np.float64)[:, None]).T
    s = np.ones(P)
    if homogeneous:
        s = np.sum(x * x, axis=1)
        with np.errstate(divide="ignore"):
            x = x * np.where(s > 0, 1.0 / np.sqrt(np.where(s > 0, s, 1.0)), 0.0)[:, None]
    x = r(x)
    z1 = x @ W1.T + d["b1"]
    h1 = r(np.maximum(z1, 0))
    z2 = h1 @ W2.T + d["b2"]
    h2 = r(np.maximum(z2, 0))
    y = h2 @ W3.T + d["b3"]
    Y = (y[:, :6] * s[:, None] / np.asarray(t_scale, np.float64)).T
    if clark_ell > 0:
        Y = Y + clark_stress(np.asarray(X, np.float64), clark_ell)
    return Y, dict(x=x, h1=h1, h2=h2, y=y, W2=W2, W3=W3, s=s)


def mlp_loss_grad(params, X, T, in_scale, t_scale, emulate_bf16=False, homogeneous=False):
    """loss = sum_p sum_o (s_p y_po - t_scale_o T_op)^2 / P and its gradient (NPARAM,)."""
    _, c = mlp_forward(params, X, in_scale, t_scale, emulate_bf16, homogeneous)
    r = bf16 if emulate_bf16 else (lambda v: v)
    P = X.shape[1]
    tgt = np.zeros((P, 8))
    tgt[:, :6] = (np.asarray(T, np.float64) * np.asarray(t_scale, np.float64)[:, None]).T
    diff = c["y"] * c["s"][:, None] - tgt
    diff[:, 6:] = 0.0
    loss = float(np.sum(diff ** 2))
    dy = r(2.0 * diff * c["s"][:, None] / P)
    dh2 = r((dy @ c["W3"]) * (c["h2"] > 0))
    dh1 = r((dh2 @ c["W2"]) * (c["h1"] > 0))
    g = {"W3": dy.T @ c["h2"], "b3": dy.sum(0), "W2": dh2.T @ c["h1"], "b2": dh2.sum(0),
         "W1": dh1.T @ c["x"], "b1": dh1.sum(0)}
    return loss, mlp_pack(g)


def adam_step(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    p = params - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v


def clark_stress(A, ell):
    """Gradient model tau_ij = ell^2/12 sum_k A_ik A_jk for A (nd*nd, P) (component i*nd+j);
    returns the nd(nd+1)/2 components in the order 00 11 22 01 02 12."""
    nd = int(round(np.sqrt(A.shape[0])))
    c = ell * ell / 12.0
    out = []
    for i in range(nd):
        out.append(c * sum(A[i * nd + k] * A[i * nd + k] for k in range(nd)))
    for i in range(nd):
        for j in range(i + 1, nd):
            out.append(c * sum(A[i * nd + k] * A[j * nd + k] for k in range(nd)))
    return np.stack(out)


def flux_from_stress(tau, A):
    """Pi = -tau_ij S_ij with tau in the compact order and A (nd*nd, P)."""
    nd = int(round(np.sqrt(A.shape[0])))
    pi = np.zeros(A.shape[1:])
    q = 0
    for i in range(nd):
        pi -= tau[q] * A[i * nd + i]
        q += 1
    for i in range(nd):
        for j in range(i + 1, nd):
            pi -= tau[q] * (A[i * nd + j] + A[j * nd + i])
            q += 1
    return pi


def coarse_graining_terms(u_phys, ks, ell, kind="gaussian"):
    """(Pi, A, tau) of the coarse-graining flux, the same formula as ``fit_oracle.coarse_graining_flux``
    (``THEORY.md:64-71``, ``src/Filters.jl:19-26``): A (nd*nd, ...) with component i*nd+j = d_j ū_i,
    tau (nd(nd+1)/2, ...) in the order 00 11 (22) 01 (02 12)."""
    from .fit_oracle import _fftn, _ifftn, filter_response
    nd = len(ks)
    ns = u_phys.shape[:nd]
    axes = tuple(range(nd))
    kc = [_kcomp(ks, d, ns) for d in range(nd)]
    G = filter_response(kind, np.sqrt(sum(k * k for k in kc)), ell)

    def filt(f):
        return np.real(_ifftn(G * _fftn(f, axes=axes), axes=axes))

    ub = [filt(u_phys[..., i]) for i in range(nd)]
    A = []
    for i in range(nd):
        bh = _fftn(ub[i], axes=axes)
        for j in range(nd):
            A.append(np.real(_ifftn(1j * kc[j] * bh, axes=axes)))
    tau = [filt(u_phys[..., i] ** 2) - ub[i] ** 2 for i in range(nd)]
    for i in range(nd):
        for j in range(i + 1, nd):
            tau.append(filt(u_phys[..., i] * u_phys[..., j]) - ub[i] * ub[j])
    A = np.stack(A)
    tau = np.stack(tau)
    return flux_from_stress(tau, A), A, tau
