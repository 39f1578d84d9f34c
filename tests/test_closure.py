"""Closure data path and learned closure: coarse-graining flux, forward spectrum, forced
Navier-Stokes evolver, BF16 tensor-core MLP (forward, gradient, Adam), gradient-model baseline.

CPU tests pin the oracle restatements (finite-difference gradient, energy budget of the evolver,
2D/3D consistency of the coarse-graining flux); GPU tests compare the library with the oracle."""
import numpy as np
import pytest

import oracle as O
from oracle import closure as OC
from fields import curl_noise_3d, solenoidal_2d, spectrum_field, e_config2

import fit_gb300 as F


def _phys(u_hat):
    nd = u_hat.ndim - 1
    Np = float(np.prod(u_hat.shape[:nd]))
    return Np * np.real(np.fft.ifftn(u_hat, axes=tuple(range(nd))))


def _energy(u_hat):
    return 0.5 * float(np.sum(np.abs(u_hat) ** 2))


# ---- oracle pins (CPU) ---------------------------------------------------------------------------

def test_oracle_mlp_gradient_finite_differences():
    rng = np.random.default_rng(4)
    p = OC.mlp_init(3).astype(np.float64)
    p[1024:1088] = rng.normal(0, 0.1, 64)   # non-zero biases
    X = rng.standard_normal((9, 37))
    T = rng.standard_normal((6, 37))
    isc, tsc = rng.uniform(0.5, 2, 9), rng.uniform(0.5, 2, 6)
    idx = [0, 5, 8, 64 * 16 - 8 + 1, 1024 + 3, 1088 + 700, 5184 + 63, 5248 + 5 * 64 + 7, 5760 + 5]
    for homog in (False, True):
        _, g = OC.mlp_loss_grad(p, X, T, isc, tsc, homogeneous=homog)
        for i in idx:
            e = np.zeros_like(p)
            e[i] = 1e-6
            lp, _ = OC.mlp_loss_grad(p + e, X, T, isc, tsc, homogeneous=homog)
            lm, _ = OC.mlp_loss_grad(p - e, X, T, isc, tsc, homogeneous=homog)
            fd = (lp - lm) / 2e-6 / X.shape[1]
            assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (homog, i, fd, g[i])
    # the padding (input columns 9..15, output rows 6..7) gets no gradient
    d = OC.mlp_unpack(g)
    assert np.all(d["W1"][:, 9:] == 0) and np.all(d["W3"][6:] == 0) and np.all(d["b3"][6:] == 0)


def test_oracle_bf16_rounding():
    v = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, 1 + 2 ** -9, -3.0, 0.0])
    assert np.array_equal(OC.bf16(v), [1.0, 1.0, 1 + 2 ** -6, 1.0, -3.0, 0.0])


def test_oracle_ns_inviscid_energy_conservation():
    """Unforced, inviscid 2/3-truncated dynamics conserve energy; SSP-RK3 keeps it to O(dt^3)."""
    ns = (16, 16, 16)
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = O.dealias_copy(spectrum_field(ns, e_config2, seed=5, project=True)[0], ns)
    u *= np.sqrt(0.5 / _energy(u))
    e0 = _energy(u)
    u1 = OC.ns_evolve(u, ks, 3, 2e-3, 0.0, 0.0, 0.0)
    assert abs(_energy(u1) - e0) <= 1e-7 * e0
    # and the state stays solenoidal and on the retained modes
    kc = [O.fit_oracle._kcomp(ks, d, ns) for d in range(3)]
    div = sum(kc[d] * u1[..., d] for d in range(3))
    assert np.abs(div).max() <= 1e-12 * np.abs(u1).max()
    assert np.all(u1[~O.keep_mask(ns)] == 0)


def test_oracle_ns_energy_budget():
    """dE/dt = power - nu * sum k^2 |û|^2 (the nonlinear term conserves energy)."""
    ns = (16, 16, 16)
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = O.dealias_copy(spectrum_field(ns, e_config2, seed=6, project=True)[0], ns)
    u *= np.sqrt(0.5 / _energy(u))
    nu, power, dt = 2e-2, 0.3, 1e-4
    kc = [O.fit_oracle._kcomp(ks, d, ns) for d in range(3)]
    k2 = sum(k * k for k in kc)
    rate = power - nu * float(np.sum(k2[..., None] * np.abs(u) ** 2))
    u1 = OC.ns_evolve(u, ks, 1, dt, nu, 2.0, power)
    assert abs((_energy(u1) - _energy(u)) / dt - rate) <= 1e-2 * abs(rate) + 1e-3 * power


def test_oracle_coarse_graining_2d_3d_consistency():
    """A 3D field independent of z with w = 0 has the 2D flux in every z plane."""
    n = 16
    ks2 = O.wavenumber_grid((n, n), (2 * np.pi,) * 2)
    ks3 = O.wavenumber_grid((n, n, 4), (2 * np.pi,) * 3)
    u2 = _phys(solenoidal_2d(n, seed=8)[0])
    u3 = np.zeros((n, n, 4, 3))
    u3[..., 0] = u2[..., 0][..., None]
    u3[..., 1] = u2[..., 1][..., None]
    for kind in ("gaussian", "sharp", "tophat"):
        p2 = O.coarse_graining_flux(u2, ks2, 0.5, kind)
        p3 = O.coarse_graining_flux(u3, ks3, 0.5, kind)
        assert np.allclose(p3, p2[..., None], rtol=0, atol=1e-12 * np.abs(p2).max())
        q, _, _ = OC.coarse_graining_terms(u2, ks2, 0.5, kind)
        assert np.allclose(q, p2, rtol=0, atol=1e-12 * np.abs(p2).max())


def test_oracle_clark_model_matches_flux_formula():
    rng = np.random.default_rng(2)
    A = rng.standard_normal((9, 11))
    tau = OC.clark_stress(A, 0.3)
    M = A.reshape(3, 3, 11)
    full = np.einsum("ikp,jkp->ijp", M, M) * 0.09 / 12
    assert np.allclose(tau[:3], [full[0, 0], full[1, 1], full[2, 2]])
    assert np.allclose(tau[3:], [full[0, 1], full[0, 2], full[1, 2]])
    S = 0.5 * (M + M.transpose(1, 0, 2))
    assert np.allclose(OC.flux_from_stress(tau, A), -np.einsum("ijp,ijp->p", full, S))


def test_coarse_graining_argument_errors():
    x = np.linspace(0, 2 * np.pi, 8, endpoint=False)
    with pytest.raises(ValueError):
        F.calculate_coarse_graining_flux((np.zeros((8, 8)),), (x, x), 0.5)
    with pytest.raises(TypeError):
        F.calculate_coarse_graining_flux((np.zeros((8, 8)),) * 2, (x, x), 0.5, filter="gaussian")


# ---- library vs oracle (GPU) ---------------------------------------------------------------------

FILTERS = {"sharp": F.SharpSpectralFilter(), "gaussian": F.GaussianFilter(), "tophat": F.TopHatFilter()}


@pytest.mark.gpu
@pytest.mark.parametrize("ns,prec,io64", [((24, 16, 8), 64, True), ((24, 16, 8), 32, True), ((24, 16, 8), 32, False),
                                          ((9, 12, 16), 32, False), ((10, 6, 12), 64, True), ((16, 16, 9), 64, True),
                                          ((64, 64, 64), 32, False)])
def test_forward_spectrum(ns, prec, io64):
    """u_hat = fft(u)/Np against numpy: fields in the compute type go straight through the z pass
    that writes the full spectrum (odd x lengths, 3 * 2^n lengths); a z length without a
    compile-time kernel (9) and mixed io/compute types take the half spectrum + scatter form."""
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
    rng = np.random.default_rng(1)
    u = rng.standard_normal(ns + (3,))
    plan = F.get_plan(ns, 3, 3, "none", prec, io64, ks)
    got = plan.forward_spectrum(u if io64 else u.astype(np.float32))
    ref = np.fft.fftn(u, axes=(0, 1, 2)) / np.prod(ns)
    tol = 1e-13 if prec == 64 else 1e-6
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["sharp", "gaussian", "tophat"])
@pytest.mark.parametrize("prec", [64, 32])
def test_coarse_graining_flux_2d(kind, prec):
    n = 32
    x = np.arange(n) * (2 * np.pi / n)
    ks = O.wavenumber_grid((n, n), (2 * np.pi,) * 2)
    u = _phys(solenoidal_2d(n, seed=11)[0])
    ell = 0.4
    res = F.calculate_coarse_graining_flux((u[..., 0], u[..., 1]), (x, x), ell, FILTERS[kind],
                                           return_diagnostics=True, precision=prec)
    Pi, A, tau = OC.coarse_graining_terms(u, ks, ell, kind)
    tol = 1e-10 if prec == 64 else 2e-5
    scale = np.abs(Pi).max()
    assert np.abs(res.flux_field - Pi).max() <= tol * scale
    assert abs(res.mean_flux - Pi.mean()) <= tol * scale
    assert np.abs(res.tau[..., 0, 1] - tau[2]).max() <= tol * np.abs(tau).max()
    assert np.abs(res.tau[..., 1, 1] - tau[1]).max() <= tol * np.abs(tau).max()
    S01 = 0.5 * (A[1] + A[2])
    assert np.abs(res.strain[..., 0, 1] - S01).max() <= tol * np.abs(A).max()


@pytest.mark.gpu
def test_coarse_graining_flux_2d_helmholtz():
    n = 32
    x = np.arange(n) * (2 * np.pi / n)
    ks = O.wavenumber_grid((n, n), (2 * np.pi,) * 2)
    rng = np.random.default_rng(3)
    u = rng.standard_normal((n, n, 2))   # not solenoidal: both parts non-zero
    res = F.calculate_coarse_graining_flux((u[..., 0], u[..., 1]), (x, x), 0.5,
                                           decomposition=F.HelmholtzDecomposition())
    uh = np.fft.fftn(u, axes=(0, 1)) / n ** 2
    parts = O.helmholtz_decompose(uh, ks)
    for name, part in parts.items():
        ref = O.coarse_graining_flux(_phys(part), ks, 0.5)
        assert np.abs(res[name].flux_field - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [64, 32])
def test_coarse_graining_flux_3d(prec):
    ns = (16, 16, 16)
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = _phys(O.dealias_copy(spectrum_field(ns, e_config2, seed=12, project=True)[0], ns))
    x = np.arange(16) * (2 * np.pi / 16)
    res = F.calculate_coarse_graining_flux(tuple(u[..., i] for i in range(3)), (x, x, x), np.pi / 4,
                                           return_diagnostics=True, precision=prec)
    Pi, A, tau = OC.coarse_graining_terms(u, ks, np.pi / 4, "gaussian")
    tol = 1e-10 if prec == 64 else 2e-5
    assert np.abs(res.flux_field - Pi).max() <= tol * np.abs(Pi).max()
    assert np.abs(res.tau[..., 1, 2] - tau[5]).max() <= tol * np.abs(tau).max()
    assert np.abs(res.strain[..., 2, 2] - A[8]).max() <= tol * np.abs(A).max()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [64, 32])
def test_forced_navier_stokes_3d(prec):
    ns = (16, 16, 16)
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = O.dealias_copy(spectrum_field(ns, e_config2, seed=13, project=True)[0], ns)
    u *= np.sqrt(0.5 / _energy(u))
    ref = OC.ns_evolve(u, ks, 4, 5e-3, 2e-3, 2.0, 0.1)
    got = F.evolve_forced_navier_stokes(u, ks, 4, 5e-3, 2e-3, kf=2.0, power=0.1, precision=prec)
    tol = 1e-11 if prec == 64 else 2e-5
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.gpu
def test_forced_navier_stokes_3d_live_box():
    """FP32 3D plans of a fused transform size evolve with the live-box nonlinear term."""
    ns = (64, 64, 64)
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = O.dealias_copy(spectrum_field(ns, e_config2, seed=17, project=True)[0], ns)
    u *= np.sqrt(0.5 / _energy(u))
    ref = OC.ns_evolve(u, ks, 3, 5e-3, 2e-3, 2.0, 0.1)
    got = F.evolve_forced_navier_stokes(u, ks, 3, 5e-3, 2e-3, kf=2.0, power=0.1, precision=32)
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()


@pytest.mark.gpu
def test_forced_navier_stokes_2d_no_dealias():
    n = 32
    ks = O.wavenumber_grid((n, n), (2 * np.pi,) * 2)
    u = solenoidal_2d(n, seed=14)[0]
    u *= np.sqrt(0.5 / _energy(u))
    ref = OC.ns_evolve(u, ks, 3, 2e-3, 1e-3, 3.0, 0.05, dealiasing="none")
    got = F.evolve_forced_navier_stokes(u, ks, 3, 2e-3, 1e-3, kf=3.0, power=0.05, dealiasing=F.NoDealiasing())
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def _mlp_case(P=1000, ld=1037, seed=0):
    rng = np.random.default_rng(seed)
    p = OC.mlp_init(seed + 1)
    p[1024:1088] = rng.normal(0, 0.05, 64).astype(np.float32)
    p[5184:5248] = rng.normal(0, 0.05, 64).astype(np.float32)
    p[5760:5766] = rng.normal(0, 0.05, 6).astype(np.float32)
    X = np.zeros((9, ld), np.float32)
    T = np.zeros((6, ld), np.float32)
    X[:, :P] = rng.standard_normal((9, P)) * rng.uniform(0.5, 3, (9, 1))
    T[:, :P] = rng.standard_normal((6, P)) * rng.uniform(0.5, 3, (6, 1))
    isc = rng.uniform(0.3, 2, 9).astype(np.float32)
    tsc = rng.uniform(0.3, 2, 6).astype(np.float32)
    return p, X, T, isc, tsc


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["tcgen05", "mma_sync"])
@pytest.mark.parametrize("homog,mixed", [(False, False), (True, False), (True, True)])
def test_mlp_forward_matches_oracle(homog, mixed, kernel, monkeypatch):
    """The forward on the fifth-generation tensor cores (default) and the warp-level mma.sync one."""
    if kernel == "mma_sync":
        monkeypatch.setenv("FIT_MLP_MMASYNC", "1")
    P, ld = 1000, 1037
    p, X, T, isc, tsc = _mlp_case(P, ld)
    m = F.SubfilterStressMLP(params=p, homogeneous=homog, mixed=mixed)
    m.ell = 0.8 if mixed else 0.0
    m.in_scale.copy_(_dev(isc))
    m.t_scale.copy_(_dev(tsc))
    Y, Pi = m.predict(_dev(X), ld, P)
    Y = Y.cpu().numpy()
    Pi = Pi.cpu().numpy()
    Ye, _ = OC.mlp_forward(p, X[:, :P], isc, tsc, emulate_bf16=True, homogeneous=homog, clark_ell=m.ell)
    Y64, _ = OC.mlp_forward(p, X[:, :P], isc, tsc, homogeneous=homog, clark_ell=m.ell)
    assert _rel(Y, Ye) <= 2e-3           # same BF16 rounding points, FP32 vs FP64 accumulation
    assert _rel(Y, Y64) <= 3e-2          # BF16 quantisation of weights, features and activations
    assert _rel(Pi, OC.flux_from_stress(Y.astype(np.float64), X[:, :P].astype(np.float64))) <= 1e-5
    assert F._lib.mlp_status() == 0


@pytest.mark.gpu
def test_mlp_forward_tcgen05_tiles():
    """tcgen05 forward on a point count that is not a multiple of its 128-point tile and on more
    tiles than CTAs (grid-stride loop), against the mma.sync forward."""
    import os
    P, ld = 300_001, 300_007
    rng = np.random.default_rng(4)
    p = OC.mlp_init(9)
    X = np.zeros((9, ld), np.float32)
    X[:, :P] = rng.standard_normal((9, P))
    m = F.SubfilterStressMLP(params=p, homogeneous=True, mixed=True)
    m.ell = 0.5
    Xd = _dev(X)
    Y, Pi = m.predict(Xd, ld, P)
    os.environ["FIT_MLP_MMASYNC"] = "1"
    try:
        Y2, Pi2 = m.predict(Xd, ld, P)
    finally:
        del os.environ["FIT_MLP_MMASYNC"]
    assert F._lib.mlp_status() == 0
    assert _rel(Y.cpu().numpy(), Y2.cpu().numpy()) <= 1e-4
    assert _rel(Pi.cpu().numpy(), Pi2.cpu().numpy()) <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["tcgen05", "mma_sync"])
@pytest.mark.parametrize("homog", [False, True])
def test_mlp_gradient_matches_oracle(homog, kernel, monkeypatch):
    """The training step on the fifth-generation tensor cores (default) and the mma.sync one."""
    if kernel == "mma_sync":
        monkeypatch.setenv("FIT_MLP_MMASYNC", "1")
    P, ld = 1000, 1037
    p, X, T, isc, tsc = _mlp_case(P, ld, seed=5)
    m = F.SubfilterStressMLP(params=p, homogeneous=homog)
    m.in_scale.copy_(_dev(isc))
    m.t_scale.copy_(_dev(tsc))
    g, loss = m.grad_of(_dev(X), _dev(T), ld, P)
    g = g.cpu().numpy().astype(np.float64)
    le, ge = OC.mlp_loss_grad(p, X[:, :P], T[:, :P], isc, tsc, emulate_bf16=True, homogeneous=homog)
    l64, g64 = OC.mlp_loss_grad(p, X[:, :P], T[:, :P], isc, tsc, homogeneous=homog)
    assert abs(float(loss.item()) - le) <= 1e-4 * le
    gd, ged, g64d = OC.mlp_unpack(g), OC.mlp_unpack(ge), OC.mlp_unpack(g64)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
        assert _rel(gd[k], ged[k]) <= 5e-3, k
        assert _rel(gd[k], g64d[k]) <= 5e-2, k
    assert np.all(gd["W1"][:, 9:] == 0) and np.all(gd["W3"][6:] == 0)
    assert F._lib.mlp_status() == 0


@pytest.mark.gpu
def test_mlp_adam_step_matches_oracle():
    import ctypes as C
    import torch
    p, X, T, isc, tsc = _mlp_case(200, 200, seed=7)
    rng = np.random.default_rng(0)
    g = rng.standard_normal(p.size).astype(np.float32)
    m0 = rng.standard_normal(p.size).astype(np.float32) * 0.1
    v0 = rng.uniform(0, 0.1, p.size).astype(np.float32)
    pd, gd, md, vd = (_dev(a) for a in (p, g, m0, v0))
    lib = F._lib.load()
    F._lib.check(lib.fit_mlp_adam(C.c_void_p(pd.data_ptr()), C.c_void_p(gd.data_ptr()), C.c_void_p(md.data_ptr()),
                                  C.c_void_p(vd.data_ptr()), 3, C.c_float(1e-3), C.c_float(0.9), C.c_float(0.999),
                                  C.c_float(1e-8), None))
    torch.cuda.synchronize()
    pr, mr, vr = OC.adam_step(p.astype(np.float64), g.astype(np.float64), m0.astype(np.float64),
                              v0.astype(np.float64), 3, 1e-3)
    assert np.abs(pd.cpu().numpy() - pr).max() <= 1e-6
    assert np.abs(md.cpu().numpy() - mr).max() <= 1e-6


@pytest.mark.gpu
def test_gradient_model_and_compare():
    import torch
    rng = np.random.default_rng(9)
    P = 3000
    A = rng.standard_normal((9, P)).astype(np.float32)
    ref = OC.flux_from_stress(OC.clark_stress(A.astype(np.float64), 0.7), A.astype(np.float64))
    data = F.ClosureData(_dev(A), None, _dev(ref), 0.7, P, 0.0)
    got = F.gradient_model_flux(data).cpu().numpy()
    assert _rel(got, ref) <= 1e-6
    b = rng.standard_normal(P)
    a = 0.5 * b + rng.standard_normal(P) * 0.1
    corr, rel = F.field_compare(_dev(a), _dev(b))
    a32, b32 = a.astype(np.float32).astype(np.float64), b.astype(np.float32).astype(np.float64)
    assert abs(corr - np.corrcoef(a32, b32)[0, 1]) <= 1e-9
    assert abs(rel - np.linalg.norm(a32 - b32) / np.linalg.norm(b32)) <= 1e-9
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_stress_residual_matches_oracle():
    import ctypes as C
    import torch
    rng = np.random.default_rng(12)
    P, ld = 777, 800
    A = np.zeros((9, ld), np.float32)
    tau = np.zeros((6, ld), np.float32)
    A[:, :P] = rng.standard_normal((9, P))
    tau[:, :P] = rng.standard_normal((6, P))
    Ad, td = _dev(A), _dev(tau)
    out = torch.zeros((6, ld), dtype=torch.float32, device="cuda")
    lib = F._lib.load()
    F._lib.check(lib.fit_stress_residual(C.c_void_p(Ad.data_ptr()), C.c_void_p(td.data_ptr()), ld, P, 0.6,
                                         C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    ref = tau[:, :P].astype(np.float64) - OC.clark_stress(A[:, :P].astype(np.float64), 0.6)
    assert _rel(out.cpu().numpy()[:, :P], ref) <= 1e-6


@pytest.mark.gpu
def test_closure_data_matches_oracle():
    import torch
    ns = (32, 32, 32)
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
    uh = O.dealias_copy(spectrum_field(ns, e_config2, seed=21, project=True)[0], ns)
    u_dev = torch.from_numpy(np.ascontiguousarray(np.moveaxis(uh, -1, 0).transpose(0, 3, 2, 1))
                             .astype(np.complex64)).cuda()
    ell = np.pi / 8
    d = F.closure_data(u_dev, ks, ell)
    Pi, A, tau = OC.coarse_graining_terms(_phys(uh.astype(np.complex64).astype(np.complex128)), ks, ell)
    n = int(np.prod(ns))
    assert _rel(d.Pi.cpu().numpy(), Pi.reshape(n, order="F")) <= 1e-4
    assert _rel(d.A.cpu().numpy(), A.transpose(0, 3, 2, 1).reshape(9, n)) <= 1e-5
    assert _rel(d.tau.cpu().numpy(), tau.transpose(0, 3, 2, 1).reshape(6, n)) <= 1e-5
    assert abs(d.mean_flux - Pi.mean()) <= 1e-4 * np.abs(Pi).max()


@pytest.mark.gpu
def test_learned_closure_gain():
    """Trained on the exact flux of half the domain of an evolved 64^3 field, the network predicts
    Pi_ell on the other half far better than the method without a closure (Pi = 0, relative
    L2 error 1) and with high correlation; the mixed form (network on the residual over the
    gradient model) beats the gradient model by at least 7 % in relative L2 error."""
    import torch
    N = 64
    ns = (N, N, N)
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
    uh = O.dealias_copy(spectrum_field(ns, e_config2, seed=31, project=True)[0], ns)
    uh *= np.sqrt(0.5 / _energy(uh))
    u_dev = torch.from_numpy(np.ascontiguousarray(np.moveaxis(uh, -1, 0).transpose(0, 3, 2, 1))
                             .astype(np.complex64)).cuda()
    F.evolve_forced_navier_stokes_device(u_dev, ks, 40, 5e-3, 2e-3, kf=2.0, power=0.1)
    d = F.closure_data(u_dev, ks, np.pi / 8)
    n = d.n
    res = {}
    for homog, mixed in ((False, False), (True, False), (True, True)):
        m = F.SubfilterStressMLP(seed=0, homogeneous=homog, mixed=mixed)
        hist = m.train(d, 0, n // 2, steps=800, batch=16384, lr=3e-3, log_every=100)
        res[(homog, mixed)] = ev = m.evaluate(d, n // 2, n)
        print(homog, mixed, hist, ev)
        assert hist[-1][1] < hist[0][1]
        assert ev["rel_l2_mlp"] < 0.6 * ev["rel_l2_no_closure"]
        assert ev["corr_mlp"] > 0.75
    # the residual network improves on the gradient model by a clear margin (measured: rel L2 0.458
    # against 0.519, 0.88x; correlation 0.853 against 0.848)
    ev = res[(True, True)]
    assert ev["rel_l2_mlp"] <= 0.93 * ev["rel_l2_gradient_model"]
    assert ev["corr_mlp"] >= ev["corr_gradient_model"] - 0.01


@pytest.mark.gpu
@pytest.mark.parametrize("ns", [(512, 8, 8), (768, 6, 4)])
def test_x_passes_long_lines_fp32(ns):
    """The real <-> half x passes at lengths whose FP32 tile is halved to 8 columns (512, 768): the
    forward spectrum against numpy, and the plain FP32 nonlinear term (its inverse x pass) against
    the FP64 plan's."""
    ks = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(ns + (3,))
    plan = F.get_plan(ns, 3, 3, "none", 32, False, ks)
    got = plan.forward_spectrum(u.astype(np.float32))
    ref = np.fft.fftn(u, axes=(0, 1, 2)) / np.prod(ns)
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()
    n32 = F.compute_nonlinear_term(ref.astype(np.complex64), ks, dealiasing=F.OrszagTwoThirds(),
                                   spectral=F.GB300Spectral(32))
    n64 = F.compute_nonlinear_term(ref, ks, dealiasing=F.OrszagTwoThirds(), spectral=F.GB300Spectral(64))
    assert np.abs(n32 - n64).max() <= 1e-5 * np.abs(n64).max()


@pytest.mark.gpu
def test_physical_to_spectral():
    """u_hat = fft(u)/Np of real physical fields through the public function, against numpy: one 2D
    field, two 2D components, four 3D FP32 fields (a chunk of three and one)."""
    rng = np.random.default_rng(8)
    u = rng.standard_normal((24, 16))
    got = F.physical_to_spectral(u)
    assert got.shape == (24, 16, 1) and got.dtype == np.complex128
    assert np.abs(got[..., 0] - np.fft.fftn(u) / u.size).max() <= 1e-13 * np.abs(np.fft.fftn(u) / u.size).max()
    v = rng.standard_normal((24, 16))
    got = F.physical_to_spectral((u, v))
    ref = np.stack([np.fft.fftn(u), np.fft.fftn(v)], axis=-1) / u.size
    assert got.shape == (24, 16, 2) and np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    w = [rng.standard_normal((16, 12, 8)).astype(np.float32) for _ in range(4)]
    got = F.physical_to_spectral(tuple(w), spectral=F.GB300Spectral(32))
    ref = np.stack([np.fft.fftn(x.astype(np.float64)) for x in w], axis=-1) / w[0].size
    assert got.shape == (16, 12, 8, 4) and got.dtype == np.complex64
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()
