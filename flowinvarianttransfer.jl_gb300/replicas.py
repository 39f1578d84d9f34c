"""Batch axis over ranks: independent inputs (snapshots of a time series, instances) distributed
round-robin over the ranks of a ``torch.distributed`` process group, each evaluated on its own
GPU with no communication during the computation, then collated in the original order or
reduced — the host-side replica runner of ``mpi_batch_map`` (``ext/FlowInvariantTransferMPIExt.jl``
``:13-68``), with ``torch.distributed`` (NCCL or gloo) in place of MPI.
"""
from __future__ import annotations


def _apply_reduction(flat, reduction):
    """``_apply_reduction`` (``ext/FlowInvariantTransferMPIExt.jl:24-36``)."""
    if reduction == "gather":
        return flat
    if reduction in ("sum", "mean"):
        acc = flat[0]
        for x in flat[1:]:
            acc = acc + x
        return acc / len(flat) if reduction == "mean" else acc
    if callable(reduction):
        acc = flat[0]
        for x in flat[1:]:
            acc = reduction(acc, x)
        return acc
    raise ValueError(f"reduce must be 'gather', 'sum', 'mean', or a binary function (got {reduction!r}).")


def mpi_batch_map(f, items, comm=None, reduce="gather", root=0):
    """``mpi_batch_map(f, items; comm, reduce=:gather, root=0)``
    (``ext/FlowInvariantTransferMPIExt.jl:39-68``).

    Rank ``r`` of ``comm`` (a ``torch.distributed`` group; default: the world) evaluates
    ``f(items[i])`` for ``i = r, r + n, r + 2n, ...`` (round-robin: balanced for similar costs and
    deterministic). The ``(i, result)`` pairs are gathered on ``root``, collated in item order and
    reduced (``"gather"`` keeps the list, ``"sum"`` / ``"mean"`` add, or a binary function folds), and
    the outcome is broadcast so every rank returns it. The process group must be initialised."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        raise ValueError("torch.distributed is not initialized; call torch.distributed.init_process_group first.")
    rank = dist.get_rank(comm)
    nproc = dist.get_world_size(comm)
    n = len(items)
    local = [(i, f(items[i])) for i in range(rank, n, nproc)]
    gathered = [None] * nproc if rank == root else None
    dist.gather_object(local, gathered, dst=dist.get_global_rank(comm, root) if comm is not None else root,
                       group=comm)
    out = [None]
    if rank == root:
        flat = [None] * n
        for chunk in gathered:                  # one chunk per rank: (index, result) pairs
            for i, res in chunk:
                flat[i] = res
        out[0] = _apply_reduction(flat, reduce)
    dist.broadcast_object_list(out, src=dist.get_global_rank(comm, root) if comm is not None else root, group=comm)
    return out[0]


batch_map = mpi_batch_map
