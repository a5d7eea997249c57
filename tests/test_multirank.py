"""The multi-GPU path (replicas over a balanced partition) exercised with gloo ranks on the
CPU; the per-rank aligner is the CPU oracle here (the host logic is what is under test)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from mhm2_staging_gb300 import sharding, workloads


@pytest.fixture(scope="module", autouse=True)
def _built(built):
    return built


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_partition_balanced_and_complete():
    p = workloads.generate(2, n=20000)
    cells = p.a_len.astype(np.int64) * p.b_len
    for world in (1, 2, 3, 8):
        parts = sharding.partition(p.a_len, p.b_len, world)
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(p.n))
        loads = [cells[q].sum() for q in parts]
        assert max(loads) - min(loads) <= cells.max()


def _worker(rank, world, port, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    from oracle import oracle

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pairs = workloads.generate(1, n=1500)
        local, idx = sharding.shard(pairs, rank, world)
        res = oracle.align_batch(local, (1, 3, 5, 2, 2), 2)
        full = sharding.gather_results(res, idx, pairs.n)
        if rank == 0:
            queue.put(full)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_equals_single_process():
    from oracle import oracle

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for pr in procs:
        pr.start()
    full = q.get(timeout=300)
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    want = oracle.align_batch(workloads.generate(1, n=1500), (1, 3, 5, 2, 2))
    assert np.array_equal(full, want)
