"""The call sequence of the Julia glue's shell-to-shell override, through the C ABI.

The reference builds ``ws.shell_idx`` for the caller's shell geometry once per workspace
(``src/Workspaces.jl:154-169``) and its mediator loop restricts and bins by it
(``src/ShellToShell/ShellToShellTransfer.jl:193-224``, ``ext/FlowInvariantTransferFFTWExt.jl:245-275``).
The glue keeps one plan per configuration in the workspace's plan bundle, installs that index with
``fit_set_shell_index`` and calls ``fit_shell_to_shell_indexed`` on every call: the first call runs
eagerly, the second captures the batched form's graph, later calls replay it. Here the same plan
is reused for three calls per geometry (isotropic, perpendicular (1,2), parallel (3,)); each result
matches the oracle: FP64 plain within 1e-11, FP32 batched within 1e-5 of max|T|. A call that bins by
edges in between replaces the table, and the next indexed call reports it (the glue re-installs).
"""
import numpy as np
import pytest

import fit_gb300 as F
import oracle as O
from fields import curl_noise_3d, e_config2, spectrum_field
from fit_gb300.plan import Plan

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [None, (1, 2), (3,)])
@pytest.mark.parametrize("form", ["fp64_plain", "fp32_batched"])
def test_indexed_shell_to_shell_reused_plan(dims, form):
    if form == "fp64_plain":
        u, ks = curl_noise_3d(12, 3)
        plan = Plan((12, 12, 12), 3, 3, "two_thirds", 64, True, ks)
        mode, tol, binning = F._lib.S2S_PLAIN, 1e-11, ("linear", 2.0)
    else:   # a fused transform size: the live-box pipeline with the caller's table
        u, ks = spectrum_field((64, 64, 64), e_config2, seed=4)
        plan = Plan((64, 64, 64), 3, 3, "two_thirds", 32, True, ks)
        mode, tol, binning = F._lib.S2S_BATCHED, 1e-5, ("linear", 6.0)
    _, edges, _, sidx = O.shell_setup(ks, binning, dims)
    nsh = len(edges) - 1
    _, _, Tref, netref, _ = O.shell_to_shell(u, ks, binning, "two_thirds", dims=dims)
    scale = np.max(np.abs(Tref))
    for _ in range(3):
        # the reference builds a new workspace, and so a new index array, on every call: installing
        # an index equal to the installed one keeps the plan's state (and its captured graph)
        plan.set_shell_index(sidx.copy(), nsh)
        T, net, asym = plan.shell_to_shell_indexed(u, nsh, 0, mode)
        assert np.max(np.abs(T - Tref)) <= tol * scale
        assert np.max(np.abs(net - netref)) <= 10 * tol * scale
        assert asym == pytest.approx(np.max(np.abs(T + T.T)), rel=1e-12, abs=1e-300)
    # an edges-based call replaces the plan's table: the indexed entry refuses until it is re-installed
    plan.spectral_flux(u, edges, F.shells.dims_mask(F.IsotropicShells(), 3), 0, 0)
    with pytest.raises(F.FitError, match="no shell index"):
        plan.shell_to_shell_indexed(u, nsh, 0, mode)
    plan.set_shell_index(sidx, nsh)
    T, _, _ = plan.shell_to_shell_indexed(u, nsh, 0, mode)
    assert np.max(np.abs(T - Tref)) <= tol * scale


def test_set_shell_index_rejects_out_of_range():
    u, ks = curl_noise_3d(8, 1)
    plan = Plan((8, 8, 8), 3, 3, "two_thirds", 64, True, ks)
    idx = np.ones((8, 8, 8), dtype=np.int64)
    idx[3, 2, 1] = 5
    with pytest.raises(ValueError, match="outside"):
        plan.set_shell_index(idx, 4)
    with pytest.raises(F.FitError, match="no shell index"):
        plan.shell_to_shell_indexed(u, 4, 0, F._lib.S2S_PLAIN)


@pytest.mark.parametrize("n,copy_engine,f64,chunks", [(64, False, False, None), (64, True, False, None),
                                                      (96, False, False, None), (64, False, True, None),
                                                      (96, False, False, (5, 3))])
def test_pinned_host_input_kept_box(n, copy_engine, f64, chunks, monkeypatch):
    """Host-pointer call of the batched 2/3 form: pinned host memory is read by the device over the
    host link (only the kept box; complex64 in 16-byte pairs with single elements at odd run ends: 64
    has an odd first run, 96 an odd start of the second; complex128 element by element), or through
    the copy engines; both match the oracle. From the second call on (mode lists current) the read
    runs in chunks of y rows beside the set-up and the first z pass (`chunks`: a chunk count that does
    not divide K + 1, on a 3-block grid); the replayed graph reads the host buffer afresh, so a new
    field written into it gives that field's matrix."""
    torch = pytest.importorskip("torch")
    if copy_engine:
        monkeypatch.setenv("FIT_KEPT_BOX_COPY_ENGINE", "1")
    if chunks:
        monkeypatch.setenv("FIT_HOST_READ_CHUNKS", str(chunks[0]))
        monkeypatch.setenv("FIT_HOST_READ_BLOCKS", str(chunks[1]))
    ns = (n, n, n)
    ct = torch.complex128 if f64 else torch.complex64
    pinned = torch.empty((3, n, n, n), dtype=ct, pin_memory=True)
    host = np.transpose(pinned.numpy(), (3, 2, 1, 0))     # column-major (n, n, n, 3) view
    u, ks = spectrum_field(ns, e_config2, seed=9)
    host[...] = u.astype(host.dtype)
    plan = Plan(ns, 3, 3, "two_thirds", 32, f64, ks)
    _, edges, Tref, _, _ = O.shell_to_shell(host.astype(np.complex128), ks, ("linear", 6.0), "two_thirds")
    before = plan.info()[8]
    for _ in range(3):
        T, _, _ = plan.shell_to_shell(host, edges, 7, 0, 0, F._lib.S2S_BATCHED)
        assert np.max(np.abs(T - Tref)) <= 1e-5 * np.max(np.abs(Tref))
    K = n // 3 - 1
    eb = 16 if f64 else 8
    assert plan.info()[8] - before == 3 * 3 * (2 * K + 1) ** 3 * eb   # only the kept box travels
    u2, _ = spectrum_field(ns, e_config2, seed=10)
    host[...] = u2.astype(host.dtype)
    _, _, Tref2, _, _ = O.shell_to_shell(host.astype(np.complex128), ks, ("linear", 6.0), "two_thirds")
    T2, _, _ = plan.shell_to_shell(host, edges, 7, 0, 0, F._lib.S2S_BATCHED)
    assert np.max(np.abs(T2 - Tref2)) <= 1e-5 * np.max(np.abs(Tref2))
    assert np.max(np.abs(Tref2 - Tref)) > 1e-3 * np.max(np.abs(Tref))


def test_pinned_host_input_separate_advecting_field():
    """Pinned host field and a separate pinned advecting field on the batched 2/3 form: the step reads
    the field's kept box in one piece before its set-up (the chunked overlap is for self-advection),
    the advecting field's kept box when the inputs are staged; eager, captured and replayed calls
    match the oracle, and only the two kept boxes travel."""
    torch = pytest.importorskip("torch")
    n = 64
    ns = (n, n, n)
    bufs = [torch.empty((3, n, n, n), dtype=torch.complex64, pin_memory=True) for _ in range(2)]
    host = [np.transpose(b.numpy(), (3, 2, 1, 0)) for b in bufs]
    u, ks = spectrum_field(ns, e_config2, seed=11)
    a, _ = spectrum_field(ns, e_config2, seed=12)
    host[0][...] = u.astype(np.complex64)
    host[1][...] = a.astype(np.complex64)
    plan = Plan(ns, 3, 3, "two_thirds", 32, False, ks)
    _, edges, Tref, _, _ = O.shell_to_shell(host[0].astype(np.complex128), ks, ("linear", 6.0), "two_thirds",
                                            adv_hat=host[1].astype(np.complex128))
    before = plan.info()[8]
    for _ in range(3):
        T, _, _ = plan.shell_to_shell(host[0], edges, 7, 0, 0, F._lib.S2S_BATCHED, adv_hat=host[1])
        assert np.max(np.abs(T - Tref)) <= 1e-5 * np.max(np.abs(Tref))
    K = n // 3 - 1
    assert plan.info()[8] - before == 3 * 2 * 3 * (2 * K + 1) ** 3 * 8
