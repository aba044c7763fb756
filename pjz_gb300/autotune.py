"""Launch-geometry autotuner for the streamed step kernels.

For a domain shape (x, y, z, PML slab total) it times a short run of each
candidate -- temporal-block depth (one or two time steps per HBM pass),
tile height, ring depth, segment length -- on the current GPU with CUDA
events and keeps the fastest per time step.  Results are cached per shape
in memory and, when ``PJZ_GB300_TUNE_CACHE`` names a file, in that JSON
file, so a batch of many problems of few shapes is tuned once per shape.
Only launch geometry changes; every candidate computes bit-identical fields.
"""

import json
import os
from typing import Dict

import numpy as np
import torch

from . import engine

_CACHE: Dict[str, dict] = {}


def _cache_path():
  return os.environ.get("PJZ_GB300_TUNE_CACHE")


def _load():
  path = _cache_path()
  if path and os.path.exists(path) and not _CACHE:
    with open(path) as f:
      _CACHE.update(json.load(f))


def _save():
  path = _cache_path()
  if path:
    with open(path, "w") as f:
      json.dump(_CACHE, f, indent=1)


def shape_key(domain, pml_widths) -> str:
  X, Y, Z = domain
  dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
  return f"{dev}|{X}x{Y}x{Z}|pml{sum(pml_widths)}"


def candidates(domain, pml_widths):
  """One step per pass: tile heights, ring depths 3-4 and the automatic or
  doubled segment length; two steps per pass: the automatic and a few
  smaller tile heights with ring depths 2-3.  Candidates whose shared
  memory does not fit are skipped when the plan is made."""
  out = []
  for stages in (3, 4):
    for tile_y in (0, 7, 10, 14, 21, 30):
      for seg_mult in (1, 2):
        out.append(dict(steps_per_pass=1, tile_y=tile_y, stages=stages,
                        seg_mult=seg_mult))
  for stages in (2, 3):
    for tile_y in (0, 8, 11, 14, 20):
      out.append(dict(steps_per_pass=2, tile_y=tile_y, stages=stages, seg_mult=1))
  return out


def tune(domain, pml_widths=(8, 8), steps: int = 40, device=None) -> dict:
  """Best launch knobs ``{steps_per_pass, tile_y, stages, seg_x}`` for this
  shape (``steps`` even, so both depths time the same steps)."""
  _load()
  key = shape_key(domain, pml_widths)
  if key in _CACHE:
    return dict(_CACHE[key])
  dev = torch.device(device or "cuda")
  X, Y, Z = domain
  lo, hi = pml_widths
  sig = np.zeros((Z, 2), np.float32)
  sig[:lo] = 1.0
  sig[Z - hi:] = 1.0
  kw = dict(domain=domain, offset=(0, 0, 0), region=domain, tt=steps + 1,
            dt=0.5, pml_widths=pml_widths, pml_kappa=np.ones((Z, 2)),
            pml_sigma=sig, pml_alpha=np.zeros((Z, 2)))
  eps = torch.full((3, X, Y, Z), 2.0, device=dev)
  mask = torch.zeros((3, X, Y), device=dev)
  best, best_ms = None, float("inf")
  for cand in candidates(domain, pml_widths):
    knob = dict(tile_y=cand["tile_y"], stages=cand["stages"], kernel=2,
                steps_per_pass=cand["steps_per_pass"])
    try:
      p = engine.Plan(**kw, **knob)
    except (ValueError, NotImplementedError):
      continue
    p.run(epsilon=eps, absorption_mask=mask, steps=(0, 1))
    auto_seg = p.launch_config()["seg_x"]
    seg = min(X, auto_seg * cand["seg_mult"])
    if cand["seg_mult"] != 1:
      p = engine.Plan(**kw, **knob, seg_x=seg)
      p.run(epsilon=eps, absorption_mask=mask, steps=(0, 1))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    p.run(epsilon=eps, absorption_mask=mask, steps=(1, steps + 1))
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    if ms < best_ms:
      cfg = p.launch_config()
      best_ms, best = ms, dict(steps_per_pass=cfg["steps_per_pass"],
                               tile_y=cfg["tile_y"], stages=cand["stages"],
                               seg_x=seg, ms_per_step=ms)
    del p
  _CACHE[key] = best
  _save()
  return dict(best)


def knobs(domain, pml_widths=(8, 8), steps: int = 40) -> Dict[str, int]:
  """Launch keyword arguments (steps_per_pass, tile_y, stages, seg_x) for
  :class:`engine.Plan` and ``LaunchParams``."""
  b = tune(domain, pml_widths, steps=steps)
  return {k: int(b[k]) for k in ("steps_per_pass", "tile_y", "stages", "seg_x")}
