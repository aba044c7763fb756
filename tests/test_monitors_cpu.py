"""Monitor boxes on the host (plan creation and monitor placement make no
CUDA call): the flat output size the library reports matches the boxes,
``Plan.split`` cuts a flat output into per-box views that cover it exactly
once, and boxes outside the domain are refused."""

import numpy as np
import pytest
import torch

from pjz_gb300 import _build, _lib, engine
from _cases import random_problem


@pytest.fixture(scope="module")
def lib():
  _build.build()
  return _lib.load()


def _plan(case, mode, **kw):
  extra = {}
  if mode == engine.OUT_PHASORS:
    n = len(range(*case["output_steps"]))
    extra["weights"] = np.random.default_rng(0).normal(size=(4, n))
  return engine.Plan(domain=case["domain"], offset=case["offset"],
                     region=case["eps"].shape[1:], tt=case["tt"], dt=case["dt"],
                     pml_widths=case["pml_widths"], pml_kappa=case["kappa"],
                     pml_sigma=case["sigma"], pml_alpha=case["alpha"],
                     source_origin=case["source_origin"],
                     source_shape=case["source_profile"].shape[2:],
                     source_ncols=case["source_profile"].shape[0],
                     output_steps=case["output_steps"], out_mode=mode, **extra, **kw)


@pytest.mark.parametrize("mode", [engine.OUT_SNAPSHOTS, engine.OUT_PHASORS])
def test_split_covers_the_flat_output(lib, mode):
  case = random_problem(3, X=20, Y=18, Z=16, pml=(3, 3), src="x", src_pos=5,
                        tt=30, steps=(10, 30, 4))
  boxes = [((0, 0, 0), (4, 5, 6)), ((10, 2, 0), (1, 12, 16)),
           ((5, 17, 0), (15, 1, 2))]
  p = _plan(case, mode, monitors=boxes)
  lead = p.num_samples if mode == engine.OUT_SNAPSHOTS else 4
  want = sum(lead * 3 * np.prod(s) for _, s in boxes)
  assert p.out_shape() == (want,)
  flat = torch.arange(want, dtype=torch.float32)
  views = p.split(flat)
  assert [tuple(v.shape) for v in views] == [(lead, 3) + s for _, s in boxes]
  joined = torch.cat([v.reshape(-1) for v in views])
  assert torch.equal(joined, flat)


def test_monitors_change_the_workspace_and_refuse_outside_boxes(lib):
  case = random_problem(4, X=20, Y=18, Z=16, pml=(3, 3), src="x", src_pos=5,
                        tt=30, steps=(10, 30, 4))
  p = _plan(case, engine.OUT_SNAPSHOTS)
  whole = p.workspace_bytes
  assert p.out_shape() == (p.num_samples, 3) + p.region
  p.set_monitors([((0, 0, 0), (2, 2, 2))])
  assert p.out_shape() == (p.num_samples * 3 * 8,)
  assert p.workspace_bytes <= whole
  with pytest.raises(ValueError, match="outside the domain"):
    p.set_monitors([((19, 0, 0), (2, 1, 1))])
