"""Replica bookkeeping across ranks, world size 2 over gloo on the CPU:
sharding covers every simulation once, timings reduce to the slowest rank,
gradient pieces sum, and a rank that fails is reported instead of hanging."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pjz_gb300 import replicas


def _free_port():
  with socket.socket() as s:
    s.bind(("127.0.0.1", 0))
    return s.getsockname()[1]


def _worker(rank, world, port, scenario, q):
  os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
  dist.init_process_group("gloo", rank=rank, world_size=world,
                          timeout=__import__("datetime").timedelta(seconds=20))
  try:
    if scenario == "ok":
      items = list(range(11))
      mine = replicas.shard(items, rank, world)
      got = [None] * world
      dist.all_gather_object(got, mine)
      t = replicas.max_over_ranks(1.0 + rank)
      g = torch.full((3, 2), float(rank + 1))
      replicas.sum_over_ranks(g)
      q.put((rank, sorted(x for part in got for x in part), t, g.tolist()))
    else:  # rank 1 fails before the barrier
      if rank == 1:
        raise RuntimeError("rank 1 failed")
      try:
        replicas.barrier(timeout_s=3.0)
        q.put((rank, "no error"))
      except Exception as e:  # noqa: BLE001
        q.put((rank, type(e).__name__))
  except RuntimeError:
    q.put((rank, "raised"))
  finally:
    if scenario == "ok":
      dist.destroy_process_group()


def _run(scenario):
  ctx = mp.get_context("spawn")
  q = ctx.Queue()
  port = _free_port()
  procs = [ctx.Process(target=_worker, args=(r, 2, port, scenario, q))
           for r in range(2)]
  for p in procs:
    p.start()
  out = [q.get(timeout=60) for _ in procs]
  for p in procs:
    p.join(timeout=60)
    if p.is_alive():
      p.kill()
  return dict((o[0], o[1:]) for o in out)


def test_shard_max_and_sum_over_two_ranks():
  res = _run("ok")
  for rank in (0, 1):
    items, t, g = res[rank]
    assert items == list(range(11))
    assert t == 2.0
    assert g == [[3.0, 3.0]] * 3


def test_failed_rank_is_reported_not_hung():
  res = _run("fail")
  assert res[1] == ("raised",)
  assert res[0][0] != "no error"


def test_shard_by_cost_balances():
  parts = replicas.shard_by_cost([5, 1, 1, 1, 1, 1], 2)
  assert sorted(i for p in parts for i in p) == list(range(6))
  loads = [sum([5, 1, 1, 1, 1, 1][i] for i in p) for p in parts]
  assert max(loads) - min(loads) <= 1


def test_shard_rejects_bad_rank():
  with pytest.raises(ValueError):
    replicas.shard([1, 2], 2, 2)
