"""Multi-GPU host logic: one process per GPU, no collective on the data path.

A single dam break does not shard without a halo exchange (the reference is single-GPU,
src/sph/sph_run.cu:117), so several GPUs run independent work: replicas of one case, or
batched instances split across ranks by instance.  The only collectives are the timing
barrier and the reductions of per-rank timings and counts.

The launcher (torchrun) sets RANK / LOCAL_RANK / WORLD_SIZE; the process group is NCCL on GPUs
and gloo on CPU (the tests).
"""
from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def partition(counts, world: int) -> list[tuple[int, int]]:
    """Split instances with particle counts `counts` into `world` contiguous blocks
    [lo, hi) of about equal particle totals; every rank gets at least one instance when there
    are as many instances as ranks."""
    n = len(counts)
    if world < 1:
        raise ValueError("world must be >= 1")
    total = float(sum(counts))
    bounds = [0]
    acc = 0.0
    i = 0
    for r in range(1, world):
        target = total * r / world
        # advance while the next instance's midpoint is below the target, leaving at least
        # one instance for each remaining rank
        while i < n - (world - r) and acc + counts[i] / 2.0 <= target:
            acc += counts[i]
            i += 1
        i = max(i, bounds[-1] + (1 if n >= world else 0))
        acc = float(sum(counts[:i]))
        bounds.append(i)
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def reduce_max(x: float) -> float:
    """Largest value over ranks (the timing rule: the slowest rank sets the step time)."""
    return _reduce(x, "max")


def reduce_sum(x: float) -> float:
    """Sum over ranks (particles processed by the whole job)."""
    return _reduce(x, "sum")


def _reduce(x: float, how: str) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if how == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def barrier() -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
