"""The S-matrix solves shared over two ranks (gloo on the CPU): the ranks'
shares cover the 2n solves exactly once, and after the exchange every rank
holds every solve's recorded boxes bit for bit as one rank holding every
solve does -- the inputs of the (device) S, objective and gradient
assembly.  The solves themselves need a GPU; here each rank fills the
recorded boxes of its own solves with seeded data (and the others with
NaN, so a missing exchange shows)."""

import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pjz_gb300 import _build, smatrix


def _problem():
  return smatrix.build_c4(domain=(80, 80, 16), tt=300, device_cells=16, edge=10,
                          monitor_inset=6, window=8, pml=3, ramp_steps=100)


def _fill(s, solves):
  for k, o in enumerate(s.outs):
    if k in solves:
      o.copy_(torch.randn(o.shape, generator=torch.Generator().manual_seed(k)))
    else:
      o.fill_(float("nan"))


def _worker(rank, world, port, q):
  os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
  dist.init_process_group("gloo", rank=rank, world_size=world,
                          timeout=__import__("datetime").timedelta(seconds=60))
  try:
    s = smatrix.SMatrixSolver(_problem(), device="cpu", rank=rank, world=world)
    _fill(s, set(s.mine))
    s.exchange()
    q.put((rank, list(s.mine), [o.numpy() for o in s.outs]))
  finally:
    dist.destroy_process_group()


def test_sharded_smatrix_assembles_like_one_rank():
  _build.build()
  one = smatrix.SMatrixSolver(_problem(), device="cpu")
  assert one.mine == list(range(len(one.plans)))
  _fill(one, set(one.mine))
  one.exchange()

  with socket.socket() as sk:
    sk.bind(("127.0.0.1", 0))
    port = sk.getsockname()[1]
  ctx = mp.get_context("spawn")
  q = ctx.Queue()
  procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
  for p in procs:
    p.start()
  out = sorted(q.get(timeout=240) for _ in procs)
  for p in procs:
    p.join(timeout=60)
    assert p.exitcode == 0
  shares = [set(o[1]) for o in out]
  assert not shares[0] & shares[1]
  assert shares[0] | shares[1] == set(range(len(one.plans)))
  for _, _, outs in out:
    for got, want in zip(outs, one.outs):
      assert np.isfinite(got).all()
      np.testing.assert_array_equal(got, want.numpy())
