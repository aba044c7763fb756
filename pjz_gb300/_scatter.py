"""pjz's ``scatter`` on the native engine (``src/pjz/_field.py:282-442``).

Same arguments and result: ``svals[i][j]`` ``(ww,)`` complex scattering
values from mode i to mode j.  Each port is one solve with the
frequency-averaged mode as source (``:354-356``); injected amplitudes and
scattering values come from the two-plane overlap with the forward/backward
wave fit (``_overlap``/``_amplitudes``, ``:293-338``), written here in torch.

Two additions to pjz's behaviour, both of which leave the values of the
default call unchanged:

* Without gradients, the solves record phasors only on the sample planes
  the overlaps read (monitor boxes of the engine, one transverse plane per
  sample position) instead of the full ``(ww, 3, xx, yy, zz)`` field, and
  all solves run together in one batched launch per time step.  The planes
  hold the same floats as the full fields would (the engine records each
  cell the same way), so the values are bit-identical to the full-field
  path; the outputs take ``O(planes)`` memory per solve.
* ``per_frequency=True`` runs one solve per (port, frequency), each with
  that frequency's mode and a single-frequency ramped sine, instead of
  pjz's single solve per port with the frequency-averaged mode (which
  excites a mixture of the modes when they differ across frequencies).

Gradients w.r.t. epsilon flow through ``field``'s adjoint (one fused adjoint
solve per solve), replacing pjz's reciprocity residuals ``f_i f_j / a_i``
(``:378-398``), whose scale its own TODO leaves open; that path keeps the
full fields, which the adjoint's dL/d-eps product needs at every voxel.
"""

from typing import Any, Sequence

import torch

from . import _field, engine
from ._field import _prop_axis, _transverse_slice, field


def _amplitudes(beta: torch.Tensor, vals: torch.Tensor, x: torch.Tensor):
  """Forward/backward wave amplitudes from samples at ``x`` (``:293-302``)."""
  bx = beta[:, None] * x[None, :].to(beta.dtype)
  a = torch.stack([torch.exp(-1j * bx), torch.exp(1j * bx)], dim=1)
  return torch.einsum("...ji,...j->...i", torch.linalg.pinv(a), vals)


def _sample_planes(pos: int, is_fwd: Any):
  """Sample positions and their wave coordinates (``:305-338``)."""
  if is_fwd is None:
    return (pos, pos), [0, 0]
  if is_fwd:
    return (pos + 1, pos + 2), [1, 2]
  return (pos - 2, pos - 1), [-2, -1]


def _overlap_from(mode, beta, pos: int, is_fwd: Any, plane, device):
  """The overlap of ``_overlap`` with ``plane(p)`` giving the transverse
  field slice at sample position ``p``."""
  beta = torch.as_tensor(beta, device=device).to(torch.complex128)
  sample_at, x = _sample_planes(pos, is_fwd)
  if is_fwd is None:
    beta = beta * 0
  elif not is_fwd:
    beta = -beta
  m = mode.to(device)
  vals = torch.stack(
      [torch.sum(m * plane(p), dim=(-4, -3, -2, -1)) for p in sample_at],
      dim=-1).to(torch.complex128)
  return _amplitudes(beta, vals, torch.tensor(x, device=device))


def _overlap(mode, beta, pos: int, is_fwd: Any, output):
  """Mode overlap at two planes next to ``pos``, split into amplitudes
  (``:305-338``)."""
  axis = _prop_axis(mode)
  return _overlap_from(mode, beta, pos, is_fwd,
                       lambda p: _transverse_slice(output, p, axis), output.device)


def _solves(modes, pos, omega, sim_params, per_frequency):
  """The solves of one scatter call: ``(port, frequency or None, source,
  source_pos, omega, sim_params)``."""
  out = []
  for i, (m, p) in enumerate(zip(modes, pos)):
    if not per_frequency:
      out.append((i, None, torch.mean(m, dim=0), p, omega, sim_params))
      continue
    for k in range(m.shape[0]):
      w = float(omega[k])
      out.append((i, k, m[k], p, [w],
                  sim_params._replace(omega_range=(w, w))))
  return out


def _planes(modes, pos, is_fwd, eps_shape):
  """Sorted ``(axis, index)`` sample planes of every port; each must lie
  inside the epsilon region."""
  planes = sorted({("xyz".index(_prop_axis(m)), s)
                   for m, p, f in zip(modes, pos, is_fwd)
                   for s in _sample_planes(p, f)[0]})
  for ax, idx in planes:
    if not 0 <= idx < eps_shape[1 + ax]:
      raise ValueError(f"sample plane {idx} along {'xyz'[ax]} lies outside "
                       f"the epsilon region (0..{eps_shape[1 + ax] - 1})")
  return planes


def _plane_phasors(epsilon, solves, planes):
  """Runs every solve in one batched launch per step, recording phasors on
  the transverse ``planes`` ``(axis, index)`` (epsilon frame) only; returns
  per solve a dict ``(axis, index) -> (ww, 3, plane)`` complex64."""
  plans, inputs = [], []
  region = tuple(int(v) for v in epsilon.shape[1:])
  for (_, _, src, p, om, sp) in solves:
    kw, om_arr = _field._setup(epsilon, _field._to_device(src, epsilon.device),
                               om, p, sp)
    off = kw["offset"]
    boxes = []
    for ax, idx in planes:
      o, s = list(off), list(region)
      o[ax] += idx
      s[ax] = 1
      boxes.append((tuple(o), tuple(s)))
    plan, prof = _field.phasor_plan(kw, om_arr, monitors=boxes, cache=False)
    plans.append((plan, om_arr.shape[0]))
    inputs.append(dict(epsilon=epsilon, absorption_mask=kw["absorption_mask"],
                       source=prof, waveform=kw["source_waveform"]))
  outs = engine.run_many([pl for pl, _ in plans], inputs)
  res = []
  for (plan, ww), (out, _) in zip(plans, outs):
    views = plan.split(out)
    res.append({pl: torch.complex(v[:ww], v[ww:]) for pl, v in zip(planes, views)})
  return res


def scatter(
    epsilon,
    omega,
    modes: Sequence[Any],
    betas: Sequence[Any],
    pos: Sequence[int],
    is_fwd: Sequence[Any],
    sim_params,
    *,
    per_frequency: bool = False,
):
  """Differentiable scattering values between ``modes`` (``:403-442``).

  Args:
    epsilon: ``(3, xx, yy, zz)`` permittivity (torch, differentiable).
    omega: ``(ww,)`` angular frequencies.
    modes: ``(ww, 2, ...)`` port modes with exactly one singular spatial axis.
    betas: ``(ww,)`` propagation constants of the modes.
    pos: port positions along their propagation axes.
    is_fwd: per port True (+ direction), False (-) or None (no fit).
    sim_params: ``SimParams``.
    per_frequency: one solve per (port, frequency) with that frequency's
      mode instead of pjz's one solve per port with the averaged mode.

  Returns:
    ``svals[i][j]``, ``(ww,)`` complex tensors.
  """
  modes = [torch.as_tensor(m) for m in modes]
  betas = [torch.as_tensor(b) for b in betas]
  solves = _solves(modes, pos, omega, sim_params, per_frequency)
  eps_t = epsilon if isinstance(epsilon, torch.Tensor) else None
  grad = torch.is_grad_enabled() and eps_t is not None and eps_t.requires_grad
  n = len(modes)
  if grad:
    fields = [field(epsilon, src, om, p, sp) for (_, _, src, p, om, sp) in solves]
    dev = fields[0].device
    slicers = [(lambda f: (lambda m, p: _transverse_slice(f, p, _prop_axis(m))))(f)
               for f in fields]
  else:
    planes = _planes(modes, pos, is_fwd, tuple(epsilon.shape))
    dev = (eps_t.device if eps_t is not None and eps_t.is_cuda
           else torch.device("cuda"))
    eps = _field._to_device(epsilon, dev).to(torch.float32)
    recorded = _plane_phasors(eps, solves, planes)

    def slicer(rec):
      def get(m, p):
        ax = "xyz".index(_prop_axis(m))
        comps = [c for c in range(3) if c != ax]
        return rec[(ax, p)][:, comps]
      return get
    slicers = [slicer(r) for r in recorded]

  def overlaps(s, k, i_src):
    """Overlaps of every port's mode with solve s (frequency k or all)."""
    get = slicers[s]
    out = []
    for j in range(n):
      m = modes[j] if k is None else modes[j][k:k + 1]
      b = betas[j] if k is None else betas[j][k:k + 1]
      out.append(_overlap_from(m, b, pos[j], is_fwd[j],
                               lambda p, m=m: get(m, p), dev))
    return out

  # svals[i][j], per frequency when solves are per (port, frequency).
  parts = [[[] for _ in range(n)] for _ in range(n)]
  for s, (i, k, *_rest) in enumerate(solves):
    ov = overlaps(s, k, i)
    amp = (torch.ones(1 if k is not None else len(betas[i]), dtype=torch.complex128,
                      device=dev) if is_fwd[i] is None else ov[i][:, 0])
    for j in range(n):
      parts[i][j].append(ov[j][:, 1] / amp)
  return [[torch.cat(parts[i][j]) for j in range(n)] for i in range(n)]
