"""Replicas over batch shards (the multi-GPU form of the stepping path).

Samples are independent time integrations (one batch element never reads
another), so N GPUs run N replicas: one process per GPU, each stepping its own
contiguous shard of the batch.  Nothing crosses ranks on the data path; only
the timing is reduced (max over ranks) and, if the caller wants them, the
results are gathered on the host.  The reference batches with jax.vmap on one
device and has no multi-device stepping of its own.
"""

from __future__ import annotations

import os


def world_from_env() -> tuple[int, int, int]:
    """(rank, local_rank, world_size) from the torchrun environment (1 process: 0, 0, 1)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, local, ws


def init(backend: str | None = None) -> tuple[int, int]:
    """Join the process group of a torchrun launch (env://; MASTER_ADDR / MASTER_PORT from the
    environment) and return (rank, world_size).  backend defaults to nccl when CUDA is available,
    else gloo.  A single process initialises nothing."""
    rank, _, ws = world_from_env()
    if ws > 1:
        import torch
        import torch.distributed as dist

        if not dist.is_initialized():
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            dist.init_process_group(backend, init_method="env://", rank=rank, world_size=ws)
    return rank, ws


def shard(per_rank: int, rank: int, start: int = 0) -> range:
    """Global sample indices (seeds) of this rank's contiguous shard."""
    return range(start + rank * per_rank, start + (rank + 1) * per_rank)


def max_over_ranks(x: float) -> float:
    """Max of a scalar (a timing) over all ranks; the identity for one process."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_to_rank0(obj):
    """Host-side gather of per-rank results (list ordered by rank on rank 0, None elsewhere)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [obj]
    out = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


def aggregate_throughput(units_per_rank: int, world_size: int, ms_per_step: float) -> float:
    """Whole-job throughput: the units all ranks processed per step over the slowest rank's time."""
    return units_per_rank * world_size / (ms_per_step * 1e-3)
