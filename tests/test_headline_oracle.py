"""The headline workload pinned to the oracle: 512^3, D = 3, the seeded k^-5/3 field of the
benchmark (seed 3), LinearBinning(14) (32 shells), OrszagTwoThirds.

Three full columns T[:, m] (mediator shells m = 1, 6, 12, 1-based: [0, 14), [70, 84), [154, 168);
the spectrum is zero above k = 170, so higher mediator shells carry no energy) of the oracle's
restatement of ``_shell_to_shell_fft!`` (``ext/FlowInvariantTransferFFTWExt.jl:238-281``, FP64, on
the complex64-rounded field the GPU forms read) against the same columns of the FP32-batched form
(within 1e-5) and the plain FP64 form (within 1e-11), in max-norm relative to max|T| over the whole
FP64 matrix. The oracle costs about a minute per column on a 16-core host.
"""
import os

import numpy as np
import pytest

import bench
import fit_gb300 as F
import oracle as O

pytestmark = pytest.mark.gpu

COLUMNS = (0, 5, 11)   # 0-based mediator shells


def test_headline_columns_match_oracle():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    F.clear_plans()
    N = 512
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = bench.make_field(N, 3, dev)
    edges = np.asarray(F.shell_edges(F.LinearBinning(14.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    assert nsh == 32
    out = {}
    for prec, mode in ((32, F._lib.S2S_BATCHED), (64, F._lib.S2S_PLAIN)):
        field = u if prec == 32 else u.to(torch.complex128)
        plan = F.Plan(ns, 3, 3, "two_thirds", prec, prec == 64, ks)
        T = torch.zeros((nsh, nsh), dtype=torch.float64, device=dev)
        plan.shell_to_shell_device(field.data_ptr(), 0, edges, 7, 0, 0, mode, T.data_ptr(), 0, 0)
        torch.cuda.synchronize()
        out[prec] = T.cpu().numpy().T          # T(n, m)
        del plan, field
        F.clear_plans()
        torch.cuda.empty_cache()
    u_np = bench.host_field(u)
    del u
    torch.cuda.empty_cache()
    O.set_fft_workers(os.cpu_count())
    try:
        st = O.s2s_setup(u_np, O.wavenumber_grid(ns, (2 * np.pi,) * 3), ("linear", 14.0), "two_thirds")
        assert np.array_equal(st["edges"], edges)
        cols = {m: O.s2s_column(st, m) for m in COLUMNS}
    finally:
        O.set_fft_workers(None)
    scale = np.max(np.abs(out[64]))
    assert 0 < scale <= 10 * max(np.max(np.abs(c)) for c in cols.values())
    for m, col in cols.items():
        assert np.max(np.abs(out[64][:, m] - col)) <= 1e-11 * scale, m
        assert np.max(np.abs(out[32][:, m] - col)) <= 1e-5 * scale, m
