"""Clock-bounded waits inside the kernels run out and the host reports it, with no GPU fault.

The bulk-copy x pass of the fused shell-to-shell pipeline and the tcgen05 MLP kernels wait on
mbarriers with a clock bound (about one second). ``FIT_TEST_WAIT_CYCLES``, a test-only setting
read at every launch, shortens the first wait on each phase to a few cycles: the wait then runs out
while the bulk copy or the tensor-core commit is still in flight. The kernel records the failure in
its device flag, waits once more on the same phase with the full bound (so no copy is still landing
and no MMA still writing when the block exits or frees its tensor memory), and the host call
returns an error naming the timeout. The next call without the setting succeeds and matches the
oracle (shell-to-shell FP32 within 1e-5 of max|T|) or the unaffected forward (MLP, bit-identical).
"""
import numpy as np
import pytest

import fit_gb300 as F
import oracle as O
from fields import e_config2, spectrum_field
from fit_gb300.plan import Plan
from oracle import closure as OC

pytestmark = pytest.mark.gpu

SHORT = "4"   # cycles: far below the latency of any bulk copy or MMA


def test_fused_x_pass_wait_runs_out(monkeypatch):
    u, ks = spectrum_field((64, 64, 64), e_config2, seed=5)
    plan = Plan((64, 64, 64), 3, 3, "two_thirds", 32, True, ks)
    _, edges, Tref, _, _ = O.shell_to_shell(u, ks, ("linear", 4.0), "two_thirds")
    monkeypatch.setenv("FIT_TEST_WAIT_CYCLES", SHORT)
    with pytest.raises(F.FitError, match="timed out"):
        plan.shell_to_shell(u, edges, 7, 0, 0, F._lib.S2S_BATCHED)
    monkeypatch.delenv("FIT_TEST_WAIT_CYCLES")
    for _ in range(3):   # eager-keyed state, then graph capture, then replay: all with the full bound
        T, _, _ = plan.shell_to_shell(u, edges, 7, 0, 0, F._lib.S2S_BATCHED)
        assert np.max(np.abs(T - Tref)) <= 1e-5 * np.max(np.abs(Tref))


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_mlp_commit_wait_runs_out(monkeypatch):
    rng = np.random.default_rng(11)
    P, ld = 4096, 4096
    p = OC.mlp_init(2)
    X = rng.standard_normal((9, ld)).astype(np.float32)
    T = rng.standard_normal((6, ld)).astype(np.float32)
    m = F.SubfilterStressMLP(params=p, homogeneous=True)
    Xd, Td = _dev(X), _dev(T)
    Y0, Pi0 = m.predict(Xd, ld, P)
    g0 = m.grad_of(Xd, Td, ld, P)[0].clone()
    assert F._lib.mlp_status() == 0
    monkeypatch.setenv("FIT_TEST_WAIT_CYCLES", SHORT)
    m.predict(Xd, ld, P)
    assert F._lib.mlp_status() == 1          # the forward's commit wait ran out and was recorded
    m.grad_of(Xd, Td, ld, P)
    assert F._lib.mlp_status() == 1          # so did the training step's
    monkeypatch.delenv("FIT_TEST_WAIT_CYCLES")
    Y1, Pi1 = m.predict(Xd, ld, P)
    g1 = m.grad_of(Xd, Td, ld, P)[0]
    assert F._lib.mlp_status() == 0
    assert np.array_equal(Y1.cpu().numpy(), Y0.cpu().numpy())
    assert np.array_equal(Pi1.cpu().numpy(), Pi0.cpu().numpy())
    assert np.allclose(g1.cpu().numpy(), g0.cpu().numpy(), rtol=1e-5, atol=1e-6)
