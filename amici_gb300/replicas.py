"""Multi-GPU execution by replicas: the instances of a batch are independent
(``amici::run_simulations`` loops over them with no exchange,
``src/amici.cpp:235-262``), so N GPUs run N contiguous shards of the batch,
one process per GPU, and the only collective is the final gather of the
per-instance results (or, for an objective, one all-reduce of llh and sllh).
"""
from __future__ import annotations

import numpy as np


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous, balanced [start, stop) of ``n`` instances for ``rank`` of
    ``world`` (the first ``n % world`` ranks take one more)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    q, r = divmod(n, world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def gather_shards(local: dict, n: int, group=None) -> dict:
    """Concatenate every rank's per-instance result arrays (instance axis
    first) into the full batch on every rank, in rank order, over
    ``torch.distributed`` (gloo or NCCL; host arrays travel as objects)."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, {k: (None if v is None else np.asarray(v)) for k, v in local.items()}, group=group)
    out = {}
    for key in local:
        vals = [p[key] for p in parts]
        out[key] = None if vals[0] is None else np.concatenate(vals, axis=0)
    for key, v in out.items():
        if v is not None and v.shape[0] != n:
            raise ValueError(f"gathered {key} has {v.shape[0]} instances, expected {n}")
    return out


def allreduce_objective(llh, sllh, group=None):
    """Sum of llh over all conditions of all ranks and of the gradients
    (one all-reduce of nplist + 1 doubles); NaN-propagating like the sum."""
    import torch
    import torch.distributed as dist

    buf = torch.tensor(np.concatenate([[np.sum(llh)], np.sum(sllh, axis=0)]), dtype=torch.float64)
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    return float(buf[0]), buf[1:].numpy()
