"""Replica aggregation of bench.py under torch.distributed: two gloo ranks on the CPU (one process
per rank, 127.0.0.1 rendezvous). Every rank runs its own copy of the workload; the whole-job value is
the units all ranks processed over the slowest rank's time, with no collective on the data path."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, ms_of_rank, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        value, ms_max = bench.replica_throughput(ws, 1.0, ms_of_rank[rank])
        bench.barrier(ws)
        q.put((rank, value, ms_max))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("ms_of_rank", [(10.0, 30.0), (25.0, 5.0)])
def test_replica_throughput_two_gloo_ranks(ms_of_rank):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, ms_of_rank, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slow = max(ms_of_rank)
    for rank, value, ms_max in out:
        assert ms_max == slow
        assert value == pytest.approx(2 * 1000.0 / slow)


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    value, ms = bench.replica_throughput(1, 3.0, 20.0)
    assert ms == 20.0 and value == pytest.approx(150.0)


def _snapshot(seed, n=12):
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from fields import kgrid
    ks = kgrid((n, n))
    kx, ky = np.meshgrid(*ks, indexing="ij")
    rng = np.random.default_rng(seed)
    psi = np.fft.fft2(rng.standard_normal((n, n))) / n ** 2
    return np.stack([1j * ky * psi, -1j * kx * psi], axis=-1), ks


def _flux_of(seed):
    sys.path.insert(0, ROOT)
    import oracle as O
    u, ks = _snapshot(seed)
    return O.spectral_flux(u, ks, ("linear", 1.0), "two_thirds")[2]


def _map_worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import numpy as np
    import torch.distributed as dist
    import __graft_entry__
    F = __graft_entry__.load_package()
    dist.init_process_group("gloo", rank=rank, world_size=ws, init_method=f"tcp://127.0.0.1:{port}")
    try:
        items = list(range(1, 6))
        g = F.mpi_batch_map(_flux_of, items)
        m = F.mpi_batch_map(_flux_of, items, reduce="mean")
        s = F.mpi_batch_map(_flux_of, items, reduce="sum")
        mx = F.mpi_batch_map(_flux_of, items, reduce=np.maximum)
        who = F.mpi_batch_map(lambda i: (i, dist.get_rank()), items)
        q.put((rank, g, m, s, mx, who))
    finally:
        dist.destroy_process_group()


def test_mpi_batch_map_two_gloo_ranks():
    """mpi_batch_map (ext/FlowInvariantTransferMPIExt.jl:39-68) as test/mpi/batch_test.jl checks it:
    gathered results in item order on every rank, mean and sum reductions, a function reduction,
    and round-robin assignment of the items to the ranks."""
    import numpy as np
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_map_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = [_flux_of(i) for i in range(1, 6)]
    for rank, g, m, s, mx, who in out:
        assert len(g) == 5 and all(np.allclose(a, b, rtol=1e-10, atol=1e-12) for a, b in zip(g, ref))
        assert np.allclose(m, sum(ref) / 5, rtol=1e-10, atol=1e-12)
        assert np.allclose(s, sum(ref), rtol=1e-10, atol=1e-12)
        assert np.allclose(mx, np.maximum.reduce(ref), rtol=1e-10, atol=1e-12)
        assert who == [(1, 0), (2, 1), (3, 0), (4, 1), (5, 0)]


def test_mpi_batch_map_needs_an_initialized_group():
    sys.path.insert(0, ROOT)
    import __graft_entry__
    F = __graft_entry__.load_package()
    with pytest.raises(ValueError):
        F.mpi_batch_map(lambda x: x, [1, 2])
