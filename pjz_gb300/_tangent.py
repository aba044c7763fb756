"""Forward-mode (tangent-linear) derivatives of ``field`` w.r.t. single voxels.

The update ``E^{n+1} = E^n + cb (curl H^{n+1/2} - J^n - sigma E^n)`` with
``cb = dt / (eps + sigma dt / 2)`` depends on a permittivity voxel only
through its own ``cb``, and ``d cb / d eps = -cb^2 / dt``.  Differentiating
one step therefore gives the same update for the tangent fields plus, at
that voxel's component only, the term
``(d cb / d eps) (curl H - J - sigma E^n) = -(cb / dt) (E^{n+1} - E^n)``.
That is exactly the engine's source term ``-cb J`` for the current
``J^n = (E^{n+1} - E^n) / dt`` (per unit change of epsilon) at the voxel.
So the directional derivative of the whole solve is one more run of the
same engine from a zero state, driven by the forward solve's own field
increments at the voxel, and projected onto phasors exactly like the
forward.  No finite difference is taken, so nothing cancels: the result
carries the FP32 rounding of an ordinary solve (about 1e-6 relative), not
the ``noise / (2 delta)`` of a central difference.

``field`` here follows ``src/pjz/_field.py:171-279``; pjz itself has no
forward-mode derivative (its ``scatter`` has a reverse-mode VJP only,
``src/pjz/_field.py:387-403``).  The voxels must be inside the epsilon
region, away from the faces that are edge-extended into the padding (each
then feeds exactly one engine cell), and off the source plane (where pjz
divides the source by epsilon, ``src/pjz/_field.py:166-167``).
"""

from typing import Sequence, Tuple

import numpy as np
import torch

from . import _field, engine


def field_voxel_jvp(epsilon, source, omega, source_pos: int,
                    sim_params: _field.SimParams,
                    voxels: Sequence[Tuple[int, int, int, int]],
                    monitor: Tuple[Tuple[int, int, int], Tuple[int, int, int]]):
  """d field / d epsilon[voxel] on a monitor box, for every voxel.

  Args:
    epsilon, source, omega, source_pos, sim_params: as for ``field``.
    voxels: ``(component, x, y, z)`` indices into ``epsilon``.
    monitor: ``(origin, shape)`` box in ``epsilon``'s frame.

  Returns:
    ``(len(voxels), ww, 3) + shape`` complex64 on epsilon's device: the
    derivative of ``field(...)[:, :, box]`` with respect to each voxel.
  """
  dev = (epsilon.device if isinstance(epsilon, torch.Tensor) and epsilon.is_cuda
         else torch.device("cuda"))
  eps = _field._to_device(epsilon, dev).to(torch.float32).detach()
  src = _field._to_device(source, dev)
  kw, om = _field._setup(eps, src, omega, source_pos, sim_params)
  mask = kw["absorption_mask"]
  domain = (int(mask.shape[1]), int(mask.shape[2]), int(kw["pml_kappa"].shape[0]))
  region = tuple(int(v) for v in eps.shape[1:])
  off = tuple(int(v) for v in kw["offset"])
  dt = float(kw["dt"])
  tt = int(kw["source_waveform"].shape[0])
  origin, shape, prof = engine.plane_source_box(kw["source_field"],
                                                kw["source_position"], domain)
  cells = []
  for v in voxels:
    c, *p = (int(t) for t in v)
    if not 0 <= c < 3:
      raise ValueError(f"voxel component {c} outside [0, 3)")
    for ax in range(3):
      edge = (p[ax] == 0 and off[ax] > 0) or (
          p[ax] == region[ax] - 1 and off[ax] + region[ax] < domain[ax])
      if not 0 <= p[ax] < region[ax] or edge:
        raise ValueError(f"voxel {tuple(v)} is outside the region or on a face "
                         "edge-extended into the padding")
    d = [p[ax] + off[ax] for ax in range(3)]
    if all(origin[ax] <= d[ax] < origin[ax] + shape[ax] for ax in range(3)):
      raise ValueError(f"voxel {tuple(v)} lies in the source box, where the "
                       "source depends on epsilon")
    cells.append((c, tuple(d)))
  (mo, ms) = monitor
  mbox = (tuple(int(o) + off[ax] for ax, o in enumerate(mo)),
          tuple(int(s) for s in ms))
  knobs = dict(_field._launch_dict(kw["launch_params"]),
               storage=_field.storage_of(kw))
  base = dict(domain=domain, offset=off, region=region, tt=tt, dt=dt,
              pml_widths=kw["pml_widths"], pml_kappa=kw["pml_kappa"],
              pml_sigma=kw["pml_sigma"], pml_alpha=kw["pml_alpha"], **knobs)

  # Forward solve recording E at the voxels after every step.
  fwd = engine.Plan(**base, source_origin=origin, source_shape=shape,
                    source_ncols=2, output_steps=(0, tt, 1),
                    out_mode=engine.OUT_SNAPSHOTS,
                    monitors=[(d, (1, 1, 1)) for _, d in cells])
  snaps, _ = fwd.run(epsilon=eps, absorption_mask=mask, source=prof,
                     waveform=kw["source_waveform"])
  series = fwd.split(snaps)  # (tt, 3, 1, 1, 1) per voxel

  weights = _field.projection_weights(om, kw["output_steps"], dt)
  unit = torch.zeros((1, 3, 1, 1, 1), dtype=torch.float32, device=dev)
  plans, inputs = [], []
  for (c, d), s in zip(cells, series):
    e = s[:, c, 0, 0, 0]
    de = e - torch.cat([e.new_zeros(1), e[:-1]])  # E after step n minus before
    wave = (de * (1.0 / dt)).reshape(tt, 1).contiguous()
    u = unit.clone()
    u[0, c] = 1.0
    plan = engine.Plan(**base, source_origin=d, source_shape=(1, 1, 1),
                       source_ncols=1, output_steps=kw["output_steps"],
                       out_mode=engine.OUT_PHASORS, weights=weights,
                       monitors=[mbox])
    plans.append(plan)
    inputs.append(dict(epsilon=eps, absorption_mask=mask, source=u,
                       waveform=wave))
  ww = om.shape[0]
  outs = engine.run_many(plans, inputs)
  res = []
  for plan, (out, _) in zip(plans, outs):
    v = plan.split(out)[0]
    res.append(torch.complex(v[:ww], v[ww:]))
  return torch.stack(res)
