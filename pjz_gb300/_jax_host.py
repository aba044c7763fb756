"""Host sides of the JAX shim's callbacks (no jax needed here).

``jax.pure_callback`` hands these functions NumPy arrays and expects NumPy
arrays back, so pjz's jitted ``field`` (``src/pjz/_field.py:171``) and its
custom VJP can call the engine from inside a trace.  They move the arrays
to the GPU, run :func:`pjz_gb300.field` (forward) or its autograd backward
(one fused adjoint solve), and return host arrays.

JAX's cotangent of a complex output is the conjugate of torch's gradient
convention (for ``L = |z|^2`` JAX gives ``2 conj(z)``, torch ``2 z``), so
the cotangent is conjugated on its way into ``torch.autograd.grad``; for a
real input both conventions agree.
"""

import numpy as np
import torch

from . import _field


def _cuda(a, dtype=None):
  t = torch.as_tensor(np.asarray(a))
  if dtype is not None:
    t = t.to(dtype)
  return t.cuda()


def field_host(epsilon, source, omega, source_pos, sim_params) -> np.ndarray:
  """``field`` on host arrays: ``(ww, 3, xx, yy, zz)`` complex64."""
  with torch.no_grad():
    out = _field.field(_cuda(epsilon, torch.float32), _cuda(source),
                       np.asarray(omega), int(source_pos), sim_params)
  return out.cpu().numpy()


def field_vjp_host(epsilon, source, omega, cotangent, source_pos,
                   sim_params) -> np.ndarray:
  """dL/d-epsilon ``(3, xx, yy, zz)`` float32 for JAX's cotangent of
  ``field``'s output: the forward is run again, then one adjoint solve."""
  e = _cuda(epsilon, torch.float32).requires_grad_(True)
  out = _field.field(e, _cuda(source), np.asarray(omega), int(source_pos),
                     sim_params)
  g = torch.conj(_cuda(cotangent).to(out.dtype))
  (ge,) = torch.autograd.grad(out, e, grad_outputs=g)
  return ge.detach().cpu().numpy().astype(np.float32)
