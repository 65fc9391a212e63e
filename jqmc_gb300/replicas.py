"""Replica-parallel bookkeeping across processes (one GPU per process).

Walkers are independent, so N GPUs run N replicas of the walker population
with no data-path collective.  Only scalars cross processes:

* timing -- a barrier and the maximum elapsed time over ranks;
* LRDMC observables per branching -- the sums (sum w, sum w/(Vd-E),
  sum w e/(Vd-E), sum w e^2/(Vd-E)) that the reference reduces over MPI ranks
  (jqmc_gfmc.py:1966-1973) are all-reduced here.

Works with any torch.distributed backend (nccl on GPUs, gloo in CPU tests).
"""

from __future__ import annotations

import torch
import torch.distributed as dist


def max_over_ranks(value: float, device=None) -> float:
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)


def sum_over_ranks(values: torch.Tensor) -> torch.Tensor:
    """All-reduce (sum) of a small tensor of per-replica sums; returns a new tensor."""
    out = values.clone()
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(out, op=dist.ReduceOp.SUM)
    return out


def lrdmc_observables(sums: torch.Tensor, num_walkers_per_rank: int):
    """(w_avg, e_L, e_L2) of one branching from the all-reduced sums."""
    tot = sum_over_ranks(sums.to(torch.float64))
    world = dist.get_world_size() if (dist.is_available() and dist.is_initialized()) else 1
    w_avg = float(tot[0]) / (num_walkers_per_rank * world)
    return w_avg, float(tot[2] / tot[1]), float(tot[3] / tot[1])
