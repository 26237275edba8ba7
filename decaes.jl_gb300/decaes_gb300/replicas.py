"""Multi-GPU runs of the path: replicas, one process per GPU.

Voxels are independent and the path has no exchange step, so N GPUs run N
independent volumes (weak scaling) with no collective on the data path.  The
only collectives are in the measurement: a barrier around the timed region
and the maximum of the ranks' times.  These helpers are backend-agnostic
(NCCL on GPUs, gloo on CPU) so the multi-rank logic is testable without GPUs.
"""
from __future__ import annotations

import os


def rank_info():
    """(world, rank, local_rank) from the launcher's environment (1, 0, 0 alone)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value: float, world: int, device: str = "cpu") -> float:
    """The maximum of a per-rank figure (the timed region's milliseconds)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_voxels_per_s(voxels_per_rank: int, ms_max: float, world: int, steps: int = 1) -> float:
    """Whole-job throughput: every rank's voxels over the slowest rank's time."""
    return world * voxels_per_rank * steps / (ms_max * 1e-3)


def replica_seed(seed: int, rank: int) -> int:
    """Each rank's volume is its own draw of the generator."""
    return seed + rank
