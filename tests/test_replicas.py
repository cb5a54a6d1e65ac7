"""Multi-process host logic of the multi-GPU path on CPU: instance partitioning and the
max/sum reductions of per-rank timings over a world_size-2 gloo process group (one process per
rank, as torchrun launches them on GPUs)."""
from __future__ import annotations

import os
import socket

import pytest


def test_partition_covers_and_balances():
    from tmp_sph_gb300.replicas import partition
    import numpy as np
    rng = np.random.default_rng(1)
    counts = [int(c) for c in rng.integers(120_000, 1_100_000, 64)]
    for world in (1, 2, 3, 4, 8, 64):
        parts = partition(counts, world)
        assert len(parts) == world
        assert parts[0][0] == 0 and parts[-1][1] == 64
        assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
        assert all(hi > lo for lo, hi in parts)
        loads = [sum(counts[lo:hi]) for lo, hi in parts]
        # balanced to within one instance of the mean
        assert max(loads) - sum(loads) / world <= max(counts)
    assert partition([5, 5], 1) == [(0, 2)]
    with pytest.raises(ValueError):
        partition([1], 0)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    from tmp_sph_gb300 import replicas
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world)})
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        ws, r, local = replicas.dist_env()
        assert (ws, r, local) == (world, rank, rank)
        replicas.barrier()
        t = replicas.reduce_max(10.0 + rank)          # per-rank "step time"
        n = replicas.reduce_sum(1000.0 * (rank + 1))  # per-rank particles
        counts = [100, 300, 200, 400]
        lo, hi = replicas.partition(counts, world)[rank]
        mine = replicas.reduce_sum(sum(counts[lo:hi]))
        out.put((rank, t, n, mine))
    finally:
        dist.destroy_process_group()


def test_gloo_world_of_two():
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, t, n, mine in res:
        assert t == 11.0          # the slowest rank's time
        assert n == 3000.0        # particles of the whole job
        assert mine == 1000.0     # every instance counted once
