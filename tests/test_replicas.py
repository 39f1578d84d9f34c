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
