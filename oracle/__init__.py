"""CPU oracle for the transfer hot path — TEST INFRASTRUCTURE ONLY.

This package restates, in FP64 numpy, the reference algorithms that the CUDA library replaces
(jbphyswx/FlowInvariantTransfer.jl v0.1.0). It exists to check the GPU results and to time a
CPU baseline. Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it; the product package never does.

Parity status: the reference ships no numeric golden vectors and its Julia toolchain is absent,
so the oracle is pinned *relationally*: its FFT path is checked against its own direct-sum
restatement (``oracle.direct``), and against every known-answer property the reference's own
test suite asserts (``test/runtests.jl``; see ``tests/test_oracle.py`` for the list).
"""
from .fit_oracle import *  # noqa: F401,F403
