"""Multi-GPU: independent scenes sharded across ranks (one process per GPU).

Scenes never interact, so the step has no exchange: rank r steps the scenes
k with k % world == r on its own GPU, and the only communication is the host-side
timing reduction (the slowest rank defines the wall time, every rank's particle-steps
add up).  A single scene does not shard (it would need a halo exchange); it runs as
independent replicas.  torch.distributed is used for the barrier and the reductions
(NCCL on GPUs, gloo on CPUs).
"""
from __future__ import annotations


def shard(items, rank: int, world: int):
    """The items rank `rank` of `world` owns: every world-th item starting at rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    return [x for k, x in enumerate(items) if k % world == rank]


def aggregate(ms: float, units: float, device=None):
    """Whole-job throughput over ranks: (max ms over ranks, sum of units over ranks,
    units per second).  Without an initialised process group it is the local value."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms, units, units / (ms / 1e3)
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item()), float(u.item()) / (float(t.item()) / 1e3)
