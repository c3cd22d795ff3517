"""Multi-GPU layout of the path: one process per GPU, grains partitioned across ranks.

The grains are test particles: given the massive bodies' stage positions they are
independent, so every rank integrates a contiguous shard of the grains together with a
full replica of the massive set (which is integrated redundantly and identically on
every rank).  No data moves between ranks during a step.  Images and SEDs are sums over
grains, so the whole system's image is the sum of the ranks' images: one all-reduce of
n_img * xsize * ysize doubles per output (n_wav doubles for an SED).
"""
from __future__ import annotations

import numpy as np

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")


def shard_range(n_dust: int, rank: int, world: int) -> tuple[int, int]:
    """Grain range [g0, g1) of `rank`: contiguous, sizes differing by at most one."""
    if not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(n_dust, world)
    g0 = rank * base + min(rank, extra)
    return g0, g0 + base + (1 if rank < extra else 0)


def shard_state(state: dict, n_grav: int, rank: int, world: int) -> dict:
    """The rank's state arrays: every massive body, then its grain shard."""
    n_dust = len(state["x"]) - n_grav
    g0, g1 = shard_range(n_dust, rank, world)
    return {k: np.concatenate([state[k][:n_grav], state[k][n_grav + g0:n_grav + g1]]) for k in FIELDS}


def gather_grains(parts: list[dict], n_grav: int) -> dict:
    """Inverse of shard_state over all ranks (massive bodies from rank 0)."""
    return {k: np.concatenate([parts[0][k][:n_grav]] + [p[k][n_grav:] for p in parts]) for k in FIELDS}


def sum_over_ranks(t, group=None):
    """All-reduce sum of an image or SED tensor (in place); no-op in a single process."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


def job_rate(units: float, seconds: float, device=None) -> tuple[float, float, float]:
    """Whole-job throughput: (sum of the ranks' units, max of their times, ratio).  The
    slowest rank sets the job's time."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return units, seconds, units / seconds
    u = torch.tensor([units], dtype=torch.float64, device=device)
    s = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    return float(u.item()), float(s.item()), float(u.item()) / float(s.item())
