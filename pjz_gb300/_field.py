"""pjz's ``field`` on the native engine: time-harmonic E fields.

Mirrors ``src/pjz/_field.py:12-279``: the same ``SimParams`` (same fields,
same defaults), the same private helpers under the same names, the same
pre-processing (z padding, ramped-sine waveform, sampling interval, source
division by epsilon, padding and even-position bump, absorption mask, z-PML
profiles) and the same output ``(ww, 3, xx, yy, zz)`` complex64.  The one
change is where the phasor projection happens: pjz records ``2ww+1`` E
snapshots and applies ``pinv(P^T)`` afterwards (``:271-279``); here the
weights are applied inside the time loop (compensated FP32 sums), so no
snapshot is stored.  The helpers are host-side set-up of a few KB.
"""

from typing import Any, NamedTuple, Tuple

import numpy as np
import torch

from . import _adjoint, engine
from ._fdtdz import LaunchParams, cached_plan, launch_knobs, _key_array


class SimParams(NamedTuple):
  """Simulation parameters; fields and defaults of ``_field.py:12-53``."""
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


def _zz(pml_widths, use_reduced_precision, launch_params=None):
  """z extent of the domain (``_field.py:56-58``); ``LaunchParams.zz`` wins."""
  knobs = launch_knobs(launch_params)
  if knobs.zz > 0:
    return knobs.zz
  return (128 if use_reduced_precision else 64) - sum(pml_widths)


def _pad_zz(epsilon_zz, pml_widths, use_reduced_precision, launch_params=None):
  """z padding (bottom, top) that fills the domain (``_field.py:61-66``)."""
  zz = _zz(pml_widths, use_reduced_precision, launch_params)
  bot = (zz - epsilon_zz) // 2
  top = zz - epsilon_zz - bot
  if bot < 0 or top < 0:
    raise ValueError(f"epsilon has {epsilon_zz} z cells, more than the "
                     f"domain's {zz}")
  return (bot, top)


def _absorption_profiles(numcells, width, smoothness):
  """1D quadratic absorber profile (``_field.py:69-76``), ``(2, numcells)``."""
  center = (numcells - 1) / 2
  pos = np.arange(numcells)[None, :] + np.array([[0.0], [0.5]])
  pos = np.clip(np.abs(pos - center) - center + width, 0, None)
  return smoothness * np.power(pos, 2)


def _cross_profiles(x, y):
  """Max of two 1D profiles over the x-y plane (``_field.py:79-81``)."""
  return np.maximum(*np.meshgrid(x, y, indexing="ij"))[None, ...]


def _absorption_mask(xx, yy, width, smoothness):
  """``(3, xx, yy)`` absorber conductivity (``_field.py:84-90``)."""
  x = _absorption_profiles(xx, width, smoothness)
  y = _absorption_profiles(yy, width, smoothness)
  return np.concatenate([_cross_profiles(x[0], y[1]),
                         _cross_profiles(x[1], y[0]),
                         _cross_profiles(x[1], y[1])])


def _safe_div(x, y):
  """Division where divide-by-zero yields 0 (``_field.py:93-95``)."""
  return np.zeros_like(x) if y == 0 else x / y


def _pml_sigma(pml_widths, zz, ln_R, m):
  """``(zz, 2)`` z-PML conductivity (``_field.py:98-106``)."""
  z = np.arange(zz)[None, :] + np.array([[0.0], [0.5]])
  z = np.stack([_safe_div(pml_widths[0] - z, pml_widths[0]),
                _safe_div(z + 0.5 - zz + pml_widths[1], pml_widths[1])],
               axis=-1)
  z = np.max(np.clip(z, 0, None), axis=-1)
  return ((m + 1) * ln_R * z**m).T


def _ramped_sin(omega, width, delay, dt, tt):
  """Frequency-averaged ramped complex sinusoid (``_field.py:109-113``)."""
  omega = np.atleast_1d(np.asarray(omega, np.float64))
  t = omega[:, None] * dt * np.arange(tt)
  waveforms = ((1 + np.tanh(t / width - delay)) / 2) * np.exp(1j * t)
  return np.mean(waveforms, axis=0)


def _sampling_interval(omega_min: float, omega_max: float, omega_n: int,
                       dt: float) -> int:
  """Sample spacing resolving ``omega_n`` frequencies (``_field.py:116-139``)."""
  period = 4 * np.pi / (omega_max + omega_min) / dt
  if omega_n == 1:
    return int(round(period / 4))
  cutoff = np.pi * (omega_n - 1) / omega_n / (omega_max - omega_min) / dt
  m = np.floor((cutoff - period / 4) / (period / 2))
  return int(round(period / 4 + m * period / 2))


def _output_phases(omega, output_steps, dt):
  """``[cos; -sin]`` phase matrix ``(2ww, ns)`` (``_field.py:142-150``)."""
  omega = np.asarray(omega, np.float64)
  theta = omega[:, None] * dt * np.arange(*output_steps)
  return np.concatenate([np.cos(theta), -np.sin(theta)], axis=0)


def _prop_axis(mode):
  """Axis whose extent is 1 (``_field.py:282-290``)."""
  shape = tuple(mode.shape[-3:])
  if shape.count(1) == 1:
    return "xyz"[shape.index(1)]
  raise ValueError(
      f"``mode.shape[-3:]`` must contain exactly one value of ``1``, "
      f"instead got ``mode.shape == {tuple(mode.shape)}``.")


def _transverse_slice(arr, pos, axis):
  """Transverse components of ``arr`` at ``pos`` (``_field.py:153-163``)."""
  a = "xyz".find(axis)
  comps = [i for i in range(3) if i != a]
  arr = arr[..., comps, :, :, :]
  return arr.narrow(arr.dim() - 3 + a, pos, 1)


def _source(mode, pos, epsilon):
  """Mode divided by epsilon at the source plane (``_field.py:166-167``)."""
  return mode / _transverse_slice(epsilon, pos, _prop_axis(mode))


def _to_device(a, device):
  if isinstance(a, torch.Tensor):
    return a.to(device)
  return torch.as_tensor(np.asarray(a)).to(device)


def _setup(epsilon, source, omega, source_pos, sim_params):
  """pjz's pre-processing (``_field.py:193-269``) -> engine arguments."""
  (omega_range, tt, dt, source_ramp, source_delay, absorption_padding,
   absorption_coeff, pml_widths, pml_alpha_coeff, pml_sigma_lnr, pml_sigma_m,
   use_z_as_batch, use_reduced_precision, launch_params) = sim_params
  dev = epsilon.device
  omega = np.atleast_1d(np.asarray(
      omega.detach().cpu().numpy() if isinstance(omega, torch.Tensor) else omega,
      np.float64))
  ww = omega.shape[0]
  pad_zz = _pad_zz(epsilon.shape[3], pml_widths, use_reduced_precision,
                   launch_params)
  padding = ((absorption_padding, absorption_padding),
             (absorption_padding, absorption_padding), pad_zz)

  rsin = _ramped_sin(omega, source_ramp, source_delay, dt, tt)
  if source.shape[3] == 1:
    waveform = np.stack([np.imag(rsin), np.real(rsin)], axis=-1)
  else:
    waveform = np.pad(np.imag(rsin)[:, None], ((0, 0), (0, 1)))

  interval = _sampling_interval(omega_range[0], omega_range[1], ww, dt)
  output_steps = (tt - 2 * interval * ww - 1, tt, interval)

  src = _source(source, source_pos, epsilon)
  for i in range(3):
    if src.shape[i + 1] == 1:
      source_pos += padding[i][0]
    else:
      src = _pad_axis(src, i + 1, padding[i])

  if (src.shape[1] == 1 or src.shape[2] == 1) and source_pos % 2 == 1:
    source_pos += 1
    waveform = np.flip(waveform, axis=1)
  elif src.shape[3] == 1:
    re = src.real if torch.is_complex(src) else src
    im = src.imag if torch.is_complex(src) else torch.zeros_like(src)
    src = torch.stack([im, re])
  if torch.is_complex(src):
    src = src.real  # fdtdz takes a real source field

  absorption_mask = _absorption_mask(epsilon.shape[1] + 2 * absorption_padding,
                                     epsilon.shape[2] + 2 * absorption_padding,
                                     absorption_padding, absorption_coeff)
  zz = _zz(pml_widths, use_reduced_precision, launch_params)
  if use_z_as_batch:
    pml_kappa = np.inf * np.ones((zz, 2))
    pml_sigma = np.zeros_like(pml_kappa)
    pml_alpha = np.zeros_like(pml_kappa)
  else:
    pml_sigma = _pml_sigma(pml_widths, zz, pml_sigma_lnr, pml_sigma_m)
    pml_kappa = np.ones_like(pml_sigma)
    pml_alpha = pml_alpha_coeff * np.ones_like(pml_sigma)

  return dict(
      epsilon=epsilon, dt=dt, source_field=src.to(torch.float32),
      source_waveform=torch.as_tensor(np.ascontiguousarray(waveform),
                                      dtype=torch.float32, device=dev),
      source_position=int(source_pos),
      absorption_mask=torch.as_tensor(absorption_mask, dtype=torch.float32,
                                      device=dev),
      pml_kappa=pml_kappa.astype(np.float32),
      pml_sigma=pml_sigma.astype(np.float32),
      pml_alpha=pml_alpha.astype(np.float32), pml_widths=tuple(pml_widths),
      output_steps=output_steps, use_reduced_precision=use_reduced_precision,
      launch_params=launch_params,
      offset=(padding[0][0], padding[1][0], padding[2][0])), omega


def _pad_axis(t, axis, pad):
  """Zero-pads tensor ``t`` by ``pad=(lo, hi)`` along ``axis``."""
  lo, hi = pad
  shape = list(t.shape)
  shape[axis] = t.shape[axis] + lo + hi
  out = torch.zeros(shape, dtype=t.dtype, device=t.device)
  out.narrow(axis, lo, t.shape[axis]).copy_(t)
  return out


def projection_weights(omega, output_steps, dt):
  """``pinv(P^T)`` of ``_field.py:276-278`` in float64: ``(2ww, ns)``."""
  return np.linalg.pinv(_output_phases(omega, output_steps, dt).T)


def phasor_plan(kw, omega, out_mode=engine.OUT_PHASORS, record_h=False,
                monitors=None, cache=True):
  """PHASORS plan for the engine arguments ``kw`` of :func:`_setup`, cached
  by its static configuration unless ``cache`` is False; ``monitors``
  (domain-frame ``(origin, shape)`` boxes) replaces the recorded region."""
  eps = kw["epsilon"]
  mask = kw["absorption_mask"]
  domain = (int(mask.shape[1]), int(mask.shape[2]), int(kw["pml_kappa"].shape[0]))
  origin, shape, prof = engine.plane_source_box(
      kw["source_field"], kw["source_position"], domain)
  tt = int(kw["source_waveform"].shape[0])
  weights = projection_weights(omega, kw["output_steps"], kw["dt"])
  knobs = launch_knobs(kw["launch_params"])
  storage = storage_of(kw)
  region = tuple(int(v) for v in eps.shape[1:])
  key = ("field", domain, region, kw["offset"], tt, float(kw["dt"]), origin,
         shape, kw["output_steps"], kw["pml_widths"],
         _key_array(kw["pml_kappa"]), _key_array(kw["pml_sigma"]),
         _key_array(kw["pml_alpha"]), weights.tobytes(), bool(record_h),
         knobs, None if monitors is None else tuple(map(tuple, monitors)),
         storage)
  make = lambda: engine.Plan(
      domain=domain, offset=kw["offset"], region=region, tt=tt, dt=kw["dt"],
      pml_widths=kw["pml_widths"], pml_kappa=kw["pml_kappa"],
      pml_sigma=kw["pml_sigma"], pml_alpha=kw["pml_alpha"],
      source_origin=origin, source_shape=shape, source_ncols=2,
      output_steps=kw["output_steps"], out_mode=out_mode, weights=weights,
      record_h=record_h, tile_y=knobs.tile_y, seg_x=knobs.seg_x,
      steps_per_pass=knobs.steps_per_pass, kernel=knobs.kernel,
      stages=knobs.stages, warps=knobs.warps, monitors=monitors,
      storage=storage)
  plan = cached_plan(key, make) if cache else make()
  return plan, prof


def storage_of(kw):
  """Engine storage for pjz's ``use_reduced_precision`` (``_field.py:52``):
  fdtdz's reduced precision is 16-bit storage, so True selects binary16
  fields with FP32 arithmetic, False FP32 throughout."""
  return engine.STORAGE_F16 if kw["use_reduced_precision"] else engine.STORAGE_F32


def _launch_dict(launch_params):
  k = launch_knobs(launch_params)
  return dict(tile_y=k.tile_y, seg_x=k.seg_x, steps_per_pass=k.steps_per_pass,
              kernel=k.kernel, stages=k.stages, warps=k.warps)


class _FieldFn(torch.autograd.Function):
  """``field`` with a fused adjoint backward (no time history).

  Forward runs over the whole domain with epsilon edge-extended (what the
  engine does outside the region anyway) so that the backward sees every
  cell an epsilon voxel feeds; backward runs one adjoint solve, adds the
  source-plane term of pjz's source division by epsilon, and folds the
  domain gradient back onto the region.
  """

  @staticmethod
  def forward(ctx, epsilon, source, omega, source_pos, sim_params):
    kw, om = _setup(epsilon, source, omega, source_pos, sim_params)
    mask = kw["absorption_mask"]
    domain = (int(mask.shape[1]), int(mask.shape[2]), int(kw["pml_kappa"].shape[0]))
    offset = kw["offset"]
    region = tuple(int(v) for v in epsilon.shape[1:])
    eps_dom = _adjoint.extend_epsilon(epsilon.detach(), domain, offset)
    kw_dom = dict(kw, epsilon=eps_dom, offset=(0, 0, 0))
    plan, prof = phasor_plan(kw_dom, om)
    out, _ = plan.run(epsilon=eps_dom, absorption_mask=mask, source=prof,
                      waveform=kw["source_waveform"])
    ww = om.shape[0]
    F = torch.complex(out[:ww], out[ww:])
    ctx.save_for_backward(F, eps_dom)
    ctx.kw = kw
    ctx.omega = om
    ctx.prof = prof
    ctx.domain, ctx.region, ctx.offset = domain, region, offset
    ctx.sim_params = sim_params
    sl = tuple(slice(o, o + s) for o, s in zip(offset, region))
    return F[(slice(None), slice(None)) + sl].contiguous()

  @staticmethod
  def backward(ctx, g_region):
    F, eps_dom = ctx.saved_tensors
    kw, om, sp = ctx.kw, ctx.omega, ctx.sim_params
    dt = float(kw["dt"])
    X, Y, Z = ctx.domain
    ww = om.shape[0]
    g = torch.zeros((ww, 3, X, Y, Z), dtype=torch.complex64, device=F.device)
    sl = tuple(slice(o, o + s) for o, s in zip(ctx.offset, ctx.region))
    g[(slice(None), slice(None)) + sl] = g_region.to(torch.complex64)
    weights = projection_weights(om, kw["output_steps"], dt)
    # pjz divides the source by epsilon at the source plane (_field.py:219).
    origin, shape, prof = engine.plane_source_box(
        kw["source_field"], kw["source_position"], ctx.domain)
    wph = _adjoint.waveform_phasors(kw["source_waveform"].cpu().numpy(),
                                    kw["output_steps"], om, dt, weights)
    wt = _adjoint.discrete_omega(om, dt)
    coef = torch.as_tensor(1j * wt * np.exp(-1.5j * om * dt), dtype=torch.complex64,
                           device=F.device)
    wphs = torch.as_tensor(wph, dtype=torch.complex64, device=F.device)
    bsl = tuple(slice(o, o + s) for o, s in zip(origin, shape))
    jh = torch.einsum("kcxyz,kw->wcxyz", prof.to(torch.complex64), wphs)
    src_term = torch.zeros_like(g)
    src_term[(slice(None), slice(None)) + bsl] = (
        coef[:, None, None, None, None] * jh / eps_dom[(slice(None),) + bsl])
    grad = _adjoint.run_adjoint(
        g=g, F=F, omega=om, dt=dt, tt=int(sp.tt), ramp_width=sp.source_ramp,
        ramp_delay=sp.source_delay, weights=weights,
        output_steps=kw["output_steps"], epsilon_domain=eps_dom,
        absorption_mask=kw["absorption_mask"], pml_widths=kw["pml_widths"],
        pml_kappa=kw["pml_kappa"], pml_sigma=kw["pml_sigma"],
        pml_alpha=kw["pml_alpha"], src_term=src_term,
        launch=dict(_launch_dict(kw["launch_params"]), storage=storage_of(kw)))
    return _adjoint.fold_to_region(grad, ctx.region, ctx.offset), None, None, None, None


def field(
    epsilon,
    source,
    omega,
    source_pos: int,
    sim_params: SimParams,
):
  """Time-harmonic solution of Maxwell's equations (``_field.py:171-279``).

  Args:
    epsilon: ``(3, xx, yy, zz)`` permittivity (CUDA tensor, or array-like).
    source: ``(2, 1, yy, zz)``, ``(2, xx, 1, zz)`` or ``(2, xx, yy, 1)``.
    omega: ``(ww,)`` angular frequencies.
    source_pos: position of the source along its propagation axis.
    sim_params: :class:`SimParams`.

  Returns:
    ``(ww, 3, xx, yy, zz)`` complex64 fields at ``omega`` on epsilon's device.
    Differentiable w.r.t. ``epsilon`` (one fused adjoint solve per backward).
  """
  dev = (epsilon.device if isinstance(epsilon, torch.Tensor) and epsilon.is_cuda
         else torch.device("cuda"))
  epsilon = _to_device(epsilon, dev).to(torch.float32)
  source = _to_device(source, dev)
  if torch.is_grad_enabled() and epsilon.requires_grad:
    return _FieldFn.apply(epsilon, source, omega, source_pos, sim_params)
  kw, omega = _setup(epsilon, source, omega, source_pos, sim_params)
  plan, prof = phasor_plan(kw, omega)
  out, _ = plan.run(epsilon=epsilon, absorption_mask=kw["absorption_mask"],
                    source=prof, waveform=kw["source_waveform"])
  ww = omega.shape[0]
  return torch.complex(out[:ww], out[ww:])
