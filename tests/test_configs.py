"""The benchmark configurations as GPU tests, each on its stated spectrum and binning (fields from
the benchmark's own seeded generators):

* 2a: 256^3, E ~ k^4 exp(-2(k/8)^2), LinearBinning(7) (32 shells), PaddedThreeHalves (384^3): the
  FP32-batched T(n,m) against the plain FP64 path (whole matrix, 1e-5 of max|T|), and the column of
  the energy-containing mediator shell [7, 14) against the oracle (FP64 within 1e-11, FP32 within
  1e-5 of max|T|; the spectrum falls by ~200 decades across the box, so the high shells' columns
  hold values near 1e-42 whose errors only mean something against max|T|);
* 2b: 32^3 resolved S(k|p) with FP64 products, shell-summed on the device, against the plain FP64
  T(n,m) of the same field (1e-11 of max|T|);
* 3: 512^3 helical partial fluxes of kinetic energy and helicity, k^-5/3 spectrum,
  DyadicBinning(2) (8 bands), the one-pass FP32 form against the per-invariant FP64 path (1e-5);
* 4: the 64-instance drawn batch, one graph launch in FP32, against the same set in FP64
  (1e-5 of each instance's max|T| and max|Pi|).
"""
import os

import numpy as np
import pytest

import bench
import fit_gb300 as F
import oracle as O

pytestmark = pytest.mark.gpu


def _torch():
    return pytest.importorskip("torch")


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def test_config2a_padded_256():
    torch = _torch()
    dev = torch.device("cuda", 0)
    F.clear_plans()
    N = 256
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = bench.make_field(N, 5, dev, spectrum="k4exp8")
    edges = np.asarray(F.shell_edges(F.LinearBinning(7.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    assert nsh == 32
    out = {}
    for prec, mode in ((32, F._lib.S2S_BATCHED), (64, F._lib.S2S_PLAIN)):
        field = u if prec == 32 else u.to(torch.complex128)
        plan = F.Plan(ns, 3, 3, "three_halves", prec, prec == 64, ks)
        T = torch.zeros((nsh, nsh), dtype=torch.float64, device=dev)
        plan.shell_to_shell_device(field.data_ptr(), 0, edges, 7, 0, 0, mode, T.data_ptr(), 0, 0)
        torch.cuda.synchronize()
        out[prec] = T.cpu().numpy().T          # T(n, m)
        del plan, field
        F.clear_plans()
        torch.cuda.empty_cache()
    assert _rel(out[32], out[64]) <= 1e-5
    # one column against the oracle (FP64 on the complex64-rounded field, 384^3 padded transforms)
    O.set_fft_workers(os.cpu_count())
    try:
        st = O.s2s_setup(bench.host_field(u), O.wavenumber_grid(ns, (2 * np.pi,) * 3), ("linear", 7.0),
                         "three_halves")
        assert np.array_equal(st["edges"], edges)
        m = 1
        col = O.s2s_column(st, m)
    finally:
        O.set_fft_workers(None)
    scale = np.max(np.abs(out[64]))
    assert 0 < scale <= 10 * np.max(np.abs(col))
    assert np.max(np.abs(out[64][:, m] - col)) <= 1e-11 * scale
    assert np.max(np.abs(out[32][:, m] - col)) <= 1e-5 * scale


def test_config2b_mode_to_mode_shell_sums_32():
    torch = _torch()
    dev = torch.device("cuda", 0)
    F.clear_plans()
    N = 32
    ns = (N, N, N)
    nm = N ** 3
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = bench.make_field(N, 5, dev, spectrum="k4exp8").to(torch.complex128).contiguous()
    plan = F.Plan(ns, 3, 3, "two_thirds", 64, True, ks)
    S = torch.empty((nm, nm), dtype=torch.float64, device=dev)     # S[p][k]: column-major [k, p]
    net = torch.empty(nm, dtype=torch.float64, device=dev)
    plan.mode_to_mode_device(u.data_ptr(), 0, True, S.data_ptr(), net.data_ptr())
    edges = np.asarray(F.shell_edges(F.LinearBinning(1.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    sid = torch.from_numpy(plan.assign_shells(edges, 7, False).ravel(order="F")).to(dev)
    A = torch.zeros((nm, nsh + 1), dtype=torch.float64, device=dev).index_add_(1, sid, S)   # A[p][n]
    B = torch.zeros((nsh + 1, nsh + 1), dtype=torch.float64, device=dev).index_add_(0, sid, A)   # B[m][n]
    Tsum = B[1:, 1:].cpu().numpy().T        # T(n, m) = sum_{k in n, p in m} S(k|p)
    # net(k) = sum_p S(k|p), as the kernel reduces it
    assert float((S.sum(dim=0) - net).abs().max()) <= 1e-12 * float(net.abs().max())
    del S, A
    T = torch.zeros((nsh, nsh), dtype=torch.float64, device=dev)
    plan.shell_to_shell_device(u.data_ptr(), 0, edges, 7, 0, 0, F._lib.S2S_PLAIN, T.data_ptr(), 0, 0)
    torch.cuda.synchronize()
    T = T.cpu().numpy().T
    assert np.max(np.abs(Tsum - T)) <= 1e-11 * np.max(np.abs(T))
    torch.cuda.empty_cache()


def test_config3_partial_fluxes_512_dyadic2():
    torch = _torch()
    dev = torch.device("cuda", 0)
    F.clear_plans()
    N = 512
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = bench.make_field(N, 3, dev)
    edges = np.asarray(F.shell_edges(F.DyadicBinning(2.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    assert nsh == 8
    invs = [F.KineticEnergy().code, F.Helicity().code]
    p32 = F.Plan(ns, 3, 3, "two_thirds", 32, False, ks)
    T = torch.zeros(2 * 8 * nsh, dtype=torch.float64, device=dev)
    for _ in range(3):   # eager, capture, replay
        p32.partial_fluxes_batched_device(u.data_ptr(), 1, invs, edges, 7, False, T.data_ptr())
        torch.cuda.synchronize()
        T32 = T.cpu().numpy().reshape(2, 8, nsh)
        if _ == 0:
            first = T32.copy()
        else:
            assert _rel(T32, first) <= 1e-12
    del p32
    F.clear_plans()
    torch.cuda.empty_cache()
    u64 = u.to(torch.complex128)
    p64 = F.Plan(ns, 3, 3, "two_thirds", 64, True, ks)
    Tq = torch.zeros(8 * nsh, dtype=torch.float64, device=dev)
    for j, inv in enumerate(invs):
        p64.partial_fluxes_device(u64.data_ptr(), 1, inv, edges, 7, False, Tq.data_ptr())
        torch.cuda.synchronize()
        assert _rel(T32[j], Tq.cpu().numpy().reshape(8, nsh)) <= 1e-5, inv
    del p64, u64
    F.clear_plans()
    torch.cuda.empty_cache()


def test_config4_full_batch():
    torch = _torch()
    dev = torch.device("cuda", 0)
    F.clear_plans()
    specs32, specs64, desc, _ = bench.draw_batch_instances(F, 3, 64, dev)
    assert len(desc) == 64 and {d.split(":")[1] for d in desc} == {"ke", "scalar"}
    b32 = F.SpectralFluxBatch(specs32, precision=32, n_branches=8, autotune=True)
    for _ in range(3):   # eager (autotuning), capture, replay
        b32.run()
    torch.cuda.synchronize()
    r32 = b32.results()
    b64 = F.SpectralFluxBatch(specs64, precision=64, n_branches=1, autotune=False)
    b64.run()
    torch.cuda.synchronize()
    r64 = b64.results()
    for d, a, b in zip(desc, r32, r64):
        assert _rel(a.transfer_spectrum.astype(np.float64), b.transfer_spectrum) <= 1e-5, d
        assert _rel(a.flux.astype(np.float64), b.flux) <= 1e-5, d
    b32.close()
    b64.close()
    F.autotune_enable(False)
    F.clear_plans()
    torch.cuda.empty_cache()
