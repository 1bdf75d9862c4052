"""Ensemble sharding over several GPUs, one process per GPU.

The reference runs one solver object per device on a contiguous slice of the
ensemble and collects the results on the host
(Tutorials_SingleSystem_PerThread/T8_MultiGPUSingleNode/MultiGPUSingleNode.cu:55-56).
Instances (per-thread) and systems (coupled) are independent, so there is no
exchange on the data path: each rank integrates its own contiguous range with
its own solver object on its own device, and the per-instance results are
gathered to rank 0 on the host afterwards (``gather``). Works with any
torch.distributed backend (gloo on CPU, nccl on GPUs); nothing here needs a
GPU.
"""
from __future__ import annotations

import numpy as np


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """(first, count) of rank's contiguous share of n units; the first n % world
    ranks take one unit more."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError(f"bad shard request: n={n}, rank={rank}, world={world}")
    base, extra = divmod(n, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def shard_case(case, rank: int, world: int):
    """The rank's instances of a per-thread ``workloads.Case`` as a
    stand-alone ensemble (shared parameters and options unchanged)."""
    first, count = shard_range(case.nt, rank, world)
    return case.subset(np.arange(first, first + count))


# Per-instance arrays and the axis their instances run along.
_INSTANCE_AXIS = {"td": 1, "x": 1, "t": 0, "cp": 1, "acc": 1, "acci": 1, "didx": 0, "dtime": 1, "dstate": 2,
                  "status": 0, "nacc": 0, "nrej": 0}


def gather(results: dict, group=None, dst: int = 0) -> dict | None:
    """Concatenate every rank's per-instance result arrays along the instance
    axis on rank ``dst`` (host gather of pickled numpy arrays; ranks in rank
    order, so the concatenation is the unsharded ensemble). Other ranks get
    None. Entries that are not per-instance arrays are taken from rank dst."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    parts = [None] * world if rank == dst else None
    dist.gather_object(results, parts, dst=dst, group=group)
    if rank != dst:
        return None
    out = {}
    for k, v in parts[dst].items():
        if k in _INSTANCE_AXIS and isinstance(v, np.ndarray):
            out[k] = np.concatenate([p[k] for p in parts], axis=_INSTANCE_AXIS[k])
        else:
            out[k] = v
    return out
