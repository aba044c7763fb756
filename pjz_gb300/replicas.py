"""Multi-GPU use of the engine: independent replicas, no data-path exchange.

Every simulation (a port solve, an adjoint, a member of a batch) is
independent, so several GPUs split the list of simulations and never talk
during a solve; the only collectives are host-side bookkeeping: the maximum
elapsed time for throughput, and optionally a sum of per-rank gradients
(<= design-box size) when the solves of one objective are spread out.
Ranks are launched one per GPU (torchrun, RANK / WORLD_SIZE / LOCAL_RANK).
"""

import datetime
import os
from typing import List, Sequence, TypeVar

import torch
import torch.distributed as dist

T = TypeVar("T")


def rank_world():
  """(rank, world size) from the environment or an initialised group."""
  if dist.is_available() and dist.is_initialized():
    return dist.get_rank(), dist.get_world_size()
  return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def shard(items: Sequence[T], rank: int, world: int) -> List[T]:
  """Round-robin share of ``items`` for ``rank`` (every item exactly once)."""
  if not 0 <= rank < world:
    raise ValueError(f"rank {rank} outside world size {world}")
  return list(items[rank::world])


def shard_by_cost(costs: Sequence[float], world: int) -> List[List[int]]:
  """Greedy longest-first assignment of item indices to ``world`` ranks so
  that the summed costs (e.g. cell-updates) are balanced."""
  loads = [0.0] * world
  out: List[List[int]] = [[] for _ in range(world)]
  for i in sorted(range(len(costs)), key=lambda k: -costs[k]):
    r = min(range(world), key=lambda k: loads[k])
    out[r].append(i)
    loads[r] += costs[i]
  return out


def max_over_ranks(value: float, device=None) -> float:
  """Maximum of a per-rank float (the job time is the slowest rank's)."""
  if not (dist.is_available() and dist.is_initialized()):
    return float(value)
  t = torch.tensor([float(value)], dtype=torch.float64, device=device)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  return float(t.item())


def sum_over_ranks(t: torch.Tensor) -> torch.Tensor:
  """In-place sum of a tensor over ranks (per-rank gradient pieces)."""
  if dist.is_available() and dist.is_initialized():
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
  return t


def barrier(timeout_s: float = 60.0):
  """Barrier that fails (instead of hanging) when a rank never arrives;
  gloo groups use a monitored barrier with ``timeout_s``."""
  if not (dist.is_available() and dist.is_initialized()):
    return
  if dist.get_backend() == "gloo":
    dist.monitored_barrier(timeout=datetime.timedelta(seconds=timeout_s))
  else:
    dist.barrier()
