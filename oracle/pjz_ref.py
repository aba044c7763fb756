"""NumPy restatement of pjz's simulation wrapper (test infrastructure only).

This module is part of the oracle: only ``tests/``, ``__graft_entry__.smoke``
and ``bench.py``'s CPU-baseline leg may import it, and only as the checker.
The product path (``pjz_gb300``) never imports anything under ``oracle/``.

Each function restates one helper of ``src/pjz/_field.py`` (pjz) in NumPy,
float64 unless stated, and cites the line range it follows.  The helpers that
the reference's own tests pin (absorption mask, PML sigma, sampling interval,
phasor sign, ramped sine) are checked against those golden vectors in
``tests/test_oracle_kats.py``.
"""

from typing import Any, NamedTuple, Tuple

import numpy as np


class SimParams(NamedTuple):
  """Same fields and defaults as ``SimParams`` in ``src/pjz/_field.py:12-53``."""
  omega_range: Tuple[float, float]
  tt: int
  dt: float = 0.5
  source_ramp: float = 4.0
  source_delay: float = 4.0
  absorption_padding: int = 50
  absorption_coeff: float = 1e-4
  pml_widths: Tuple[int, int] = (16, 16)
  pml_alpha_coeff: float = 0.0
  pml_sigma_lnr: float = 0.5
  pml_sigma_m: float = 1.3
  use_z_as_batch: bool = False
  use_reduced_precision: bool = True
  launch_params: Any = None


def zz_budget(pml_widths, use_reduced_precision):
  """``_zz``, ``src/pjz/_field.py:56-58``."""
  return (128 if use_reduced_precision else 64) - sum(pml_widths)


def pad_zz(epsilon_zz, pml_widths, use_reduced_precision):
  """``_pad_zz``, ``src/pjz/_field.py:61-66``."""
  zz = zz_budget(pml_widths, use_reduced_precision)
  bot = (zz - epsilon_zz) // 2
  return (bot, zz - epsilon_zz - bot)


def absorption_profiles(numcells, width, smoothness):
  """``_absorption_profiles``, ``src/pjz/_field.py:69-76``."""
  center = (numcells - 1) / 2
  pos = np.arange(numcells)[None, :] + np.array([[0.0], [0.5]])
  pos = np.clip(np.abs(pos - center) - center + width, 0, None)
  return smoothness * pos**2


def cross_profiles(x, y):
  """``_cross_profiles``, ``src/pjz/_field.py:79-81``."""
  return np.maximum(*np.meshgrid(x, y, indexing="ij"))[None, ...]


def absorption_mask(xx, yy, width, smoothness):
  """``_absorption_mask``, ``src/pjz/_field.py:84-90``: ``(3, xx, yy)``."""
  x = absorption_profiles(xx, width, smoothness)
  y = absorption_profiles(yy, width, smoothness)
  return np.concatenate([cross_profiles(x[0], y[1]),
                         cross_profiles(x[1], y[0]),
                         cross_profiles(x[1], y[1])])


def pml_sigma(pml_widths, zz, ln_R, m):
  """``_pml_sigma``, ``src/pjz/_field.py:93-106``: ``(zz, 2)``."""
  z = np.arange(zz)[None, :] + np.array([[0.0], [0.5]])

  def safe_div(a, b):
    return np.zeros_like(a) if b == 0 else a / b

  z = np.stack([safe_div(pml_widths[0] - z, pml_widths[0]),
                safe_div(z + 0.5 - zz + pml_widths[1], pml_widths[1])],
               axis=-1)
  z = np.max(np.clip(z, 0, None), axis=-1)
  return ((m + 1) * ln_R * z**m).T


def ramped_sin(omega, width, delay, dt, tt):
  """``_ramped_sin``, ``src/pjz/_field.py:109-113`` (complex, ``(tt,)``)."""
  omega = np.atleast_1d(np.asarray(omega, np.float64))
  t = omega[:, None] * dt * np.arange(tt)
  w = ((1 + np.tanh(t / width - delay)) / 2) * np.exp(1j * t)
  return np.mean(w, axis=0)


def sampling_interval(omega_min, omega_max, omega_n, dt):
  """``_sampling_interval``, ``src/pjz/_field.py:116-139``."""
  period = 4 * np.pi / (omega_max + omega_min) / dt
  if omega_n == 1:
    return int(round(period / 4))
  cutoff = np.pi * (omega_n - 1) / omega_n / (omega_max - omega_min) / dt
  m = np.floor((cutoff - period / 4) / (period / 2))
  return int(round(period / 4 + m * period / 2))


def output_steps(tt, interval, ww):
  """Output step triple of ``field``, ``src/pjz/_field.py:214-216``."""
  return (tt - 2 * interval * ww - 1, tt, interval)


def output_phases(omega, steps, dt):
  """``_output_phases``, ``src/pjz/_field.py:142-150``: ``(2ww, ns)``."""
  omega = np.asarray(omega, np.float64)
  theta = omega[:, None] * dt * np.arange(*steps)
  return np.concatenate([np.cos(theta), -np.sin(theta)], axis=0)


def projection_weights(omega, steps, dt):
  """``pinv(P^T)`` of ``src/pjz/_field.py:276-278``: ``(2ww, ns)`` float64."""
  return np.linalg.pinv(output_phases(omega, steps, dt).T)


def frequency_components(snapshots, steps, omega, dt):
  """Phasors from time samples, the projection of ``src/pjz/_field.py:271-279``.

  ``snapshots`` has the sample axis first.  Returns ``(ww, ...)`` complex with
  ``f(t) = Re(F exp(i omega dt t))``.
  """
  omega = np.asarray(omega, np.float64)
  theta = omega[:, None] * dt * np.asarray(steps, np.float64)[None, :]
  p = np.concatenate([np.cos(theta), -np.sin(theta)], axis=0)
  out = np.einsum("ij,j...->i...", np.linalg.pinv(p.T), snapshots)
  ww = omega.shape[0]
  return out[:ww] + 1j * out[ww:]


def prop_axis(mode):
  """``_prop_axis``, ``src/pjz/_field.py:282-290``."""
  shape = tuple(mode.shape[-3:])
  if shape.count(1) == 1:
    return "xyz"[shape.index(1)]
  raise ValueError(
      f"``mode.shape[-3:]`` must contain exactly one value of ``1``, "
      f"instead got ``mode.shape == {mode.shape}``.")


def transverse_slice(arr, pos, axis):
  """``_transverse_slice``, ``src/pjz/_field.py:153-163``."""
  a = "xyz".find(axis)
  comps = [i for i in range(3) if i != a]
  arr = arr[..., comps, :, :, :]
  sl = [slice(None)] * arr.ndim
  sl[arr.ndim - 3 + a] = slice(pos, pos + 1)
  return arr[tuple(sl)]


def field_setup(epsilon, source, omega, source_pos, sim_params, zz=None):
  """Pre-processing of ``field``, ``src/pjz/_field.py:193-269``.

  Returns the keyword arguments ``field`` hands to the FDTD engine (float32
  arrays, the ``fdtdz`` calling convention), plus ``omega`` for the
  projection.  ``zz`` replaces pjz's fixed z budget (``_zz``, :56-58) when
  given, since the engine under test takes any thin z extent.
  """
  sp = SimParams(*sim_params)
  epsilon = np.asarray(epsilon)
  omega = np.atleast_1d(np.asarray(omega, np.float64))
  zz = zz or zz_budget(sp.pml_widths, sp.use_reduced_precision)
  bot = (zz - epsilon.shape[3]) // 2
  pad_z = (bot, zz - epsilon.shape[3] - bot)
  ap = sp.absorption_padding
  padding = ((ap, ap), (ap, ap), pad_z)

  rsin = ramped_sin(omega, sp.source_ramp, sp.source_delay, sp.dt, sp.tt)
  if source.shape[3] == 1:
    waveform = np.stack([np.imag(rsin), np.real(rsin)], axis=-1)
  else:
    waveform = np.pad(np.imag(rsin)[:, None], ((0, 0), (0, 1)))

  interval = sampling_interval(sp.omega_range[0], sp.omega_range[1],
                               omega.shape[0], sp.dt)
  steps = output_steps(sp.tt, interval, omega.shape[0])

  src = np.asarray(source) / transverse_slice(epsilon, source_pos,
                                              prop_axis(source))
  for i in range(3):
    if src.shape[i + 1] == 1:
      source_pos += padding[i][0]
    else:
      src = np.pad(src, (i + 1) * ((0, 0),) + (padding[i],)
                   + (2 - i) * ((0, 0),))
  if (src.shape[1] == 1 or src.shape[2] == 1) and source_pos % 2 == 1:
    source_pos += 1
    waveform = np.flip(waveform, axis=1)
  elif src.shape[3] == 1:
    src = np.stack([np.imag(src), np.real(src)])

  mask = absorption_mask(epsilon.shape[1] + 2 * ap, epsilon.shape[2] + 2 * ap,
                         ap, sp.absorption_coeff)
  if sp.use_z_as_batch:
    kappa = np.inf * np.ones((zz, 2))
    sigma = np.zeros_like(kappa)
    alpha = np.zeros_like(kappa)
  else:
    sigma = pml_sigma(sp.pml_widths, zz, sp.pml_sigma_lnr, sp.pml_sigma_m)
    kappa = np.ones_like(sigma)
    alpha = sp.pml_alpha_coeff * np.ones_like(sigma)

  f32 = lambda a: np.ascontiguousarray(np.real(a), dtype=np.float32)
  return dict(
      epsilon=f32(epsilon), dt=float(sp.dt), source_field=f32(src),
      source_waveform=f32(waveform), source_position=int(source_pos),
      absorption_mask=f32(mask), pml_kappa=f32(kappa), pml_sigma=f32(sigma),
      pml_alpha=f32(alpha), pml_widths=tuple(sp.pml_widths),
      output_steps=steps, use_reduced_precision=sp.use_reduced_precision,
      launch_params=sp.launch_params,
      offset=(padding[0][0], padding[1][0], padding[2][0]),
  ), omega


def amplitudes(beta, vals, x):
  """``_amplitudes``, ``src/pjz/_field.py:293-302``."""
  beta = np.asarray(beta)
  a = np.stack([np.exp(-1j * beta[:, None] * x),
                np.exp(1j * beta[:, None] * x)], axis=1)
  return np.einsum("...ji,...j->...i", np.linalg.pinv(a), vals)


def overlap(mode, beta, pos, is_fwd, output):
  """``_overlap``, ``src/pjz/_field.py:305-338``."""
  beta = np.asarray(beta, dtype=np.complex128)
  if is_fwd is None:
    x, sample_at, beta = np.array([0, 0]), (pos, pos), beta * 0
  elif is_fwd:
    x, sample_at = np.array([1, 2]), (pos + 1, pos + 2)
  else:
    x, sample_at, beta = np.array([-2, -1]), (pos - 2, pos - 1), -beta
  ax = prop_axis(mode)
  vals = np.stack(
      [np.sum(mode * transverse_slice(output, p, ax), axis=(-4, -3, -2, -1))
       for p in sample_at], axis=-1)
  return amplitudes(beta, vals, x)
