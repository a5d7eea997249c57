"""Multi-GPU use of the aligner: replicas over a balanced pair partition.

Pairs are independent, so N GPUs run N independent driver replicas (one process per GPU,
device = rank % device_count as in the reference's GPUDriver::init, driver.cpp:220) on a
partition of the batch balanced by forward cells; results are gathered on the host.
There is no device collective on the data path.
"""
from __future__ import annotations

import numpy as np

from .driver import Pairs


def partition(a_len: np.ndarray, b_len: np.ndarray, world: int) -> list[np.ndarray]:
    """Pair indices per rank, balanced by len(A)*len(B): pairs sorted by cells (largest
    first) are dealt in a snake order 0..w-1, w-1..0, which keeps rank loads within one
    pair's cells of each other.  Each rank's indices come back in ascending order."""
    n = int(a_len.shape[0])
    if world < 1:
        raise ValueError("world must be >= 1")
    cells = a_len.astype(np.int64) * b_len.astype(np.int64)
    order = np.argsort(-cells, kind="stable")
    pos = np.arange(n)
    rnd, k = pos // world, pos % world
    owner = np.where(rnd % 2 == 0, k, world - 1 - k)
    return [np.sort(order[owner == r]) for r in range(world)]


def shard(pairs: Pairs, rank: int, world: int) -> tuple[Pairs, np.ndarray]:
    """This rank's pairs (compact batch) and their indices in the full batch."""
    idx = partition(pairs.a_len, pairs.b_len, world)[rank]
    return pairs.subset(idx), idx


def gather_results(local: np.ndarray, idx: np.ndarray, n: int, group=None) -> np.ndarray | None:
    """Gathers every rank's n_local x 5 results into the full n x 5 array on rank 0
    (host-side, through torch.distributed's object gather); other ranks get None."""
    import torch.distributed as dist

    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    parts = [None] * world if rank == 0 else None
    dist.gather_object((idx, local), parts, dst=0, group=group)
    if rank != 0:
        return None
    out = np.zeros((n, 5), dtype=np.int32)
    for i, o in parts:
        out[i] = o
    return out
