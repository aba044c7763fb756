"""Autotuner on the GPU: it returns launch knobs for a shape (temporal-block
depth, tile height, ring depth, segment length), caches them, and a plan
built with them is bit-identical to the oracle."""

import numpy as np
import pytest
import torch

import oracle
from pjz_gb300 import autotune, engine
from _cases import oracle_kwargs, random_problem

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def test_tuned_knobs_are_valid_and_exact(native, tmp_path, monkeypatch):
  monkeypatch.setenv("PJZ_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
  autotune._CACHE.clear()
  case = random_problem(70, X=40, Y=36, Z=32, pml=(4, 4), tt=30, steps=(10, 30, 3))
  k = autotune.knobs(case["domain"], case["pml_widths"], steps=8)
  assert k["steps_per_pass"] in (1, 2) and k["tile_y"] > 0 and k["seg_x"] > 0
  assert (tmp_path / "tune.json").exists()
  assert autotune.knobs(case["domain"], case["pml_widths"]) == k  # cached
  p = engine.Plan(domain=case["domain"], offset=case["offset"],
                  region=case["eps"].shape[1:], tt=case["tt"], dt=case["dt"],
                  pml_widths=case["pml_widths"], pml_kappa=case["kappa"],
                  pml_sigma=case["sigma"], pml_alpha=case["alpha"],
                  source_origin=case["source_origin"],
                  source_shape=case["source_profile"].shape[2:],
                  source_ncols=case["source_profile"].shape[0],
                  output_steps=case["output_steps"], out_mode=engine.OUT_SNAPSHOTS,
                  kernel=2, **k)
  t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=DEV)
  out, _ = p.run(epsilon=t(case["eps"]), absorption_mask=t(case["mask"]),
                 source=t(case["source_profile"]), waveform=t(case["waveform"]))
  torch.cuda.synchronize()
  assert np.array_equal(out.cpu().numpy(), oracle.run(**oracle_kwargs(case))["out"])
