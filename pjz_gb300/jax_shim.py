"""``fdtdz_jax``-compatible entry points for pjz's JAX code.

pjz imports ``fdtdz_jax`` and calls ``fdtdz_jax.fdtdz(**kw)``
(``src/pjz/_field.py:6, 254-269``).  This module offers the same call, plus
``field`` and ``scatter`` with ``jax.custom_vjp`` whose backward runs the
engine's fused adjoint, so pjz code can switch with::

    import pjz_gb300.jax_shim as fdtdz_jax

``fdtdz`` hands arrays between JAX and torch through DLPack (zero-copy on
the same GPU) when called eagerly; under ``jax.jit`` it goes through
``jax.pure_callback`` (a host round trip of the inputs and outputs).
``field``'s forward and backward always run in ``jax.pure_callback``
(``pjz_gb300/_jax_host.py``), so pjz's jitted ``field`` and ``scatter``
(``src/pjz/_field.py:171, 403-404``) can call them inside a trace; the
backward runs the forward again and then one fused adjoint solve.  jax is
not a dependency: importing this module without jax raises ImportError.
"""

try:
  import jax
  import jax.numpy as jnp
except ImportError as e:  # pragma: no cover - exercised only without jax
  raise ImportError("pjz_gb300.jax_shim needs jax") from e

from functools import partial

import numpy as np
import torch
import torch.utils.dlpack as tdl

from . import _fdtdz, _field, _jax_host


def _to_torch(x):
  if isinstance(x, jax.Array):
    try:
      return tdl.from_dlpack(x)
    except (TypeError, RuntimeError, BufferError):
      return torch.as_tensor(np.asarray(x))
  if isinstance(x, np.ndarray):
    return torch.as_tensor(x)
  return x


def _to_jax(t: torch.Tensor):
  try:
    return jax.dlpack.from_dlpack(t.contiguous())
  except (TypeError, RuntimeError, BufferError):
    return jnp.asarray(t.detach().cpu().numpy())


def _concrete(*xs):
  return not any(isinstance(x, jax.core.Tracer) for x in xs)


def fdtdz(**kw):
  """``fdtdz_jax.fdtdz`` replacement: E snapshots ``(ns, 3, xx, yy, zz)``."""
  arrays = {k: v for k, v in kw.items() if isinstance(v, (jax.Array, np.ndarray))}
  if _concrete(*arrays.values()):
    t = {k: _to_torch(v) for k, v in kw.items()}
    if not t["epsilon"].is_cuda:
      t["epsilon"] = t["epsilon"].cuda()
    return _to_jax(_fdtdz.fdtdz(**t))
  ns = len(range(*kw["output_steps"]))
  shape = (ns,) + tuple(kw["epsilon"].shape)
  static = {k: v for k, v in kw.items() if k not in arrays}

  def host(**a):
    out = _fdtdz.fdtdz(**{k: torch.as_tensor(np.asarray(v)) for k, v in a.items()},
                       **static)
    return out.cpu().numpy()

  return jax.pure_callback(host, jax.ShapeDtypeStruct(shape, jnp.float32),
                           **arrays)


@partial(jax.custom_vjp, nondiff_argnums=(3, 4))
def field(epsilon, source, omega, source_pos, sim_params):
  """pjz ``field`` on the engine; differentiable w.r.t. ``epsilon`` and
  usable under ``jax.jit`` (the engine runs in a ``jax.pure_callback``)."""
  shape = (jnp.shape(omega)[0], 3) + tuple(jnp.shape(epsilon)[1:])
  return jax.pure_callback(
      partial(_jax_host.field_host, source_pos=source_pos,
              sim_params=sim_params),
      jax.ShapeDtypeStruct(shape, jnp.complex64), epsilon, source, omega)


def _field_fwd(epsilon, source, omega, source_pos, sim_params):
  # The residuals are the inputs: the backward callback runs the forward
  # again before its adjoint solve (a traced function cannot keep torch
  # tensors between the two callbacks).
  return field(epsilon, source, omega, source_pos, sim_params), (
      epsilon, source, omega)


def _field_bwd(source_pos, sim_params, res, g):
  epsilon, source, omega = res
  ge = jax.pure_callback(
      partial(_jax_host.field_vjp_host, source_pos=source_pos,
              sim_params=sim_params),
      jax.ShapeDtypeStruct(jnp.shape(epsilon), jnp.float32), epsilon, source,
      omega, g)
  return ge, None, None


field.defvjp(_field_fwd, _field_bwd)


def _slice_jnp(arr, pos, axis):
  """Transverse components of ``arr`` at ``pos`` along ``axis`` (jnp form of
  ``_field._transverse_slice``)."""
  a = "xyz".find(axis)
  comps = [i for i in range(3) if i != a]
  arr = arr[..., jnp.asarray(comps), :, :, :]
  return jax.lax.dynamic_slice_in_dim(arr, pos, 1, axis=arr.ndim - 3 + a)


def _overlap_jnp(mode, beta, pos, is_fwd, output):
  """Two-plane overlap and forward/backward split (jnp form of
  ``_scatter._overlap`` / ``_amplitudes``)."""
  beta = jnp.asarray(beta).astype(jnp.complex64)
  if is_fwd is None:
    x, at, beta = [0, 0], (pos, pos), beta * 0
  elif is_fwd:
    x, at = [1, 2], (pos + 1, pos + 2)
  else:
    x, at, beta = [-2, -1], (pos - 2, pos - 1), -beta
  axis = _field._prop_axis(mode)
  vals = jnp.stack([jnp.sum(mode * _slice_jnp(output, p, axis),
                            axis=(-4, -3, -2, -1)) for p in at], axis=-1)
  bx = beta[:, None] * jnp.asarray(x, jnp.float32)[None, :]
  a = jnp.stack([jnp.exp(-1j * bx), jnp.exp(1j * bx)], axis=1)
  return jnp.einsum("...ji,...j->...i", jnp.linalg.pinv(a), vals)


def scatter(epsilon, omega, modes, betas, pos, is_fwd, sim_params):
  """pjz ``scatter`` (``src/pjz/_field.py:403-442``): one :func:`field` solve
  per port with the frequency-averaged mode as source, then the two-plane
  overlap fit; differentiable w.r.t. ``epsilon`` through :func:`field`'s
  custom VJP (one fused adjoint solve per port)."""
  modes = [jnp.asarray(m) for m in modes]
  fields = [field(epsilon, jnp.mean(m, axis=0), omega, p, sim_params)
            for m, p in zip(modes, pos)]
  amps = [jnp.ones(jnp.shape(b), jnp.complex64) if fwd is None
          else _overlap_jnp(m, b, p, fwd, f)[:, 0]
          for f, m, b, p, fwd in zip(fields, modes, betas, pos, is_fwd)]
  return [[_overlap_jnp(m, b, p, fwd, f)[:, 1] / a
           for m, b, p, fwd in zip(modes, betas, pos, is_fwd)]
          for a, f in zip(amps, fields)]
