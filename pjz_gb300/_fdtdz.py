"""Drop-in for ``fdtdz_jax.fdtdz``, the engine call of pjz's ``field``.

Same keyword arguments and return value as the call at
``src/pjz/_field.py:254-269``: E-field snapshots ``(ns, 3, xx, yy, zz)``
float32 at ``range(*output_steps)`` over the epsilon region, computed by the
native sm_103a engine.  Arrays are torch tensors (CUDA) or anything
``torch.as_tensor`` accepts; the result lives on epsilon's CUDA device.
"""

from typing import Any, NamedTuple, Optional, Tuple

import numpy as np
import torch

from . import engine


class LaunchParams(NamedTuple):
  """Engine knobs carried in pjz's opaque ``launch_params`` (``_field.py:53``).

  ``zz`` overrides pjz's fixed z budget of 64/128 cells (``_field.py:56-58``)
  so that any thin z extent can be simulated; 0 keeps pjz's rule.
  """
  tile_y: int = 0
  seg_x: int = 0
  steps_per_pass: int = 0
  zz: int = 0
  kernel: int = 0
  stages: int = 0
  warps: int = 0


def launch_knobs(launch_params: Any) -> LaunchParams:
  """Reads engine knobs from ``launch_params``; other forms mean "auto"."""
  if isinstance(launch_params, LaunchParams):
    return launch_params
  if isinstance(launch_params, dict):
    return LaunchParams(**{k: int(v) for k, v in launch_params.items()
                           if k in LaunchParams._fields})
  return LaunchParams()


_PLANS = {}
_MAX_PLANS = 16


def _key_array(a) -> bytes:
  if isinstance(a, torch.Tensor):
    a = a.detach().cpu().numpy()
  return np.ascontiguousarray(np.asarray(a, np.float32)).tobytes()


def cached_plan(key, factory):
  """Plans are cached by their static configuration (pjz re-jits likewise)."""
  plan = _PLANS.get(key)
  if plan is None:
    if len(_PLANS) >= _MAX_PLANS:
      _PLANS.pop(next(iter(_PLANS)))
    plan = factory()
    _PLANS[key] = plan
  return plan


def _as_device(a, device):
  if isinstance(a, torch.Tensor):
    return a.to(device)
  return torch.as_tensor(np.asarray(a)).to(device)


def fdtdz(
    epsilon,
    dt: float,
    source_field,
    source_waveform,
    source_position: int,
    absorption_mask,
    pml_kappa,
    pml_sigma,
    pml_alpha,
    pml_widths: Tuple[int, int],
    output_steps: Tuple[int, int, int],
    use_reduced_precision: bool = False,
    launch_params: Any = None,
    offset: Tuple[int, int, int] = (0, 0, 0),
    *,
    device: Optional[torch.device] = None,
) -> torch.Tensor:
  """FDTD solve with fdtdz's calling convention; returns E snapshots.

  The domain is ``absorption_mask.shape[1:]`` in x, y and
  ``pml_kappa.shape[0]`` in z; ``epsilon`` sits at ``offset`` inside it and is
  edge-extended outside.  ``use_reduced_precision`` selects binary16
  storage of the fields, coefficients and CPML state with FP32 arithmetic
  (fdtdz's 16-bit mode); False stores FP32.
  """
  dev = device or (epsilon.device if isinstance(epsilon, torch.Tensor)
                   and epsilon.is_cuda else torch.device("cuda"))
  eps = _as_device(epsilon, dev)
  mask = _as_device(absorption_mask, dev)
  sf = _as_device(source_field, dev)
  if torch.is_complex(sf):
    sf = sf.real
  wave = _as_device(source_waveform, dev).to(torch.float32)
  if eps.dim() != 4 or eps.shape[0] != 3:
    raise ValueError(f"epsilon must be (3, xx, yy, zz), got {tuple(eps.shape)}")
  if mask.dim() != 3 or mask.shape[0] != 3:
    raise ValueError("absorption_mask must be (3, xx, yy), got "
                     f"{tuple(mask.shape)}")
  zz = int(np.shape(pml_kappa)[0])
  domain = (int(mask.shape[1]), int(mask.shape[2]), zz)
  if wave.dim() != 2 or wave.shape[1] != 2:
    raise ValueError(f"source_waveform must be (tt, 2), got {tuple(wave.shape)}")
  tt = int(wave.shape[0])
  origin, shape, prof = engine.plane_source_box(sf, source_position, domain)
  knobs = launch_knobs(launch_params)
  steps = tuple(int(v) for v in output_steps)
  region = tuple(int(v) for v in eps.shape[1:])
  key = ("fdtdz", domain, region, tuple(offset), tt, float(dt), origin, shape,
         steps, tuple(pml_widths), _key_array(pml_kappa), _key_array(pml_sigma),
         _key_array(pml_alpha), knobs, bool(use_reduced_precision))
  plan = cached_plan(key, lambda: engine.Plan(
      domain=domain, offset=offset, region=region, tt=tt, dt=dt,
      pml_widths=pml_widths, pml_kappa=pml_kappa, pml_sigma=pml_sigma,
      pml_alpha=pml_alpha, source_origin=origin, source_shape=shape,
      source_ncols=2, output_steps=steps, out_mode=engine.OUT_SNAPSHOTS,
      tile_y=knobs.tile_y, seg_x=knobs.seg_x,
      steps_per_pass=knobs.steps_per_pass, kernel=knobs.kernel,
      stages=knobs.stages, warps=knobs.warps,
      storage=engine.STORAGE_F16 if use_reduced_precision else engine.STORAGE_F32))
  out, _ = plan.run(epsilon=eps, absorption_mask=mask, source=prof,
                    waveform=wave)
  return out
