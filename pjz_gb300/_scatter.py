"""pjz's ``scatter`` on the native engine (``src/pjz/_field.py:282-442``).

Same arguments and result: ``svals[i][j]`` ``(ww,)`` complex scattering
values from mode i to mode j.  Each port is one ``field`` solve with the
frequency-averaged mode as source (``:354-356``); injected amplitudes and
scattering values come from the two-plane overlap with the forward/backward
wave fit (``_overlap``/``_amplitudes``, ``:293-338``), written here in torch.
Gradients w.r.t. epsilon flow through ``field``'s adjoint (one fused adjoint
solve per port), replacing pjz's reciprocity residuals ``f_i f_j / a_i``
(``:378-398``), whose scale its own TODO leaves open.
"""

from typing import Any, Sequence

import torch

from ._field import _prop_axis, _transverse_slice, field


def _amplitudes(beta: torch.Tensor, vals: torch.Tensor, x: torch.Tensor):
  """Forward/backward wave amplitudes from samples at ``x`` (``:293-302``)."""
  bx = beta[:, None] * x[None, :].to(beta.dtype)
  a = torch.stack([torch.exp(-1j * bx), torch.exp(1j * bx)], dim=1)
  return torch.einsum("...ji,...j->...i", torch.linalg.pinv(a), vals)


def _overlap(mode, beta, pos: int, is_fwd: Any, output):
  """Mode overlap at two planes next to ``pos``, split into amplitudes
  (``:305-338``)."""
  beta = torch.as_tensor(beta, device=output.device).to(torch.complex128)
  if is_fwd is None:
    x, sample_at, beta = [0, 0], (pos, pos), beta * 0
  elif is_fwd:
    x, sample_at = [1, 2], (pos + 1, pos + 2)
  else:
    x, sample_at, beta = [-2, -1], (pos - 2, pos - 1), -beta
  axis = _prop_axis(mode)
  m = mode.to(output.device)
  vals = torch.stack(
      [torch.sum(m * _transverse_slice(output, p, axis), dim=(-4, -3, -2, -1))
       for p in sample_at], dim=-1).to(torch.complex128)
  return _amplitudes(beta, vals, torch.tensor(x, device=output.device))


def scatter(
    epsilon,
    omega,
    modes: Sequence[Any],
    betas: Sequence[Any],
    pos: Sequence[int],
    is_fwd: Sequence[Any],
    sim_params,
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

  Returns:
    ``svals[i][j]``, ``(ww,)`` complex tensors.
  """
  modes = [torch.as_tensor(m) for m in modes]
  fields = [field(epsilon, torch.mean(m, dim=0), omega, p, sim_params)
            for m, p in zip(modes, pos)]
  amplitudes = [
      torch.ones(len(torch.as_tensor(b)), dtype=torch.complex128,
                 device=f.device) if fwd is None
      else _overlap(m, b, p, fwd, f)[:, 0]
      for f, m, b, p, fwd in zip(fields, modes, betas, pos, is_fwd)]
  return [[_overlap(m, b, p, fwd, f)[:, 1] / a
           for m, b, p, fwd in zip(modes, betas, pos, is_fwd)]
          for a, f in zip(amplitudes, fields)]
