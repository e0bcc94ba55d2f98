"""Independent replicas on several GPUs of one node.

The hot path has no exchange step (points, rays and grid slabs are
independent), so N GPUs run N independent replicas, one process per GPU
launched by torch.distributed.run.  The ranks share only a barrier around
the timed region and the maximum of their step times; the whole-job
throughput is N times one replica's units over that maximum (weak scaling).
The process group is NCCL on GPUs and works the same with gloo on the CPU.
"""

from __future__ import annotations

import os

import torch


def rank_info():
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def barrier():
    d = _dist()
    if d is not None:
        d.barrier()


def max_over_ranks(value, device=None):
    """The largest ``value`` over all ranks (the value itself on one rank)."""
    d = _dist()
    if d is None:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, seconds, world):
    """Whole-job throughput of ``world`` replicas that each processed
    ``units_per_rank`` units, the slowest in ``seconds``."""
    return world * units_per_rank / seconds
