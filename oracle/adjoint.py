"""FP64 restatement of the field adjoint (test infrastructure only).

Independent NumPy restatement of the reciprocity adjoint the product uses
for ``field``'s gradient (same discrete derivation; see the docstring of the
product's adjoint module for the formulas), run on the FP64 oracle engine.
Only ``tests/`` import it.  It replaces pjz's reciprocity VJP
(``src/pjz/_field.py:378-398``), whose scale is unverified by its own TODO
(``:378``); the gradient oracle of record is central finite differences.
"""

import numpy as np

import oracle
from oracle import pjz_ref


def _pml_coeff(kappa, sigma, alpha, dt):
  """Engine CPML coefficients (ik, b, c), rounded to float32 as it uses them."""
  if np.isinf(kappa):
    return 0.0, float(np.float32(np.exp(-alpha * dt))), 0.0
  b = np.exp(-(sigma / kappa + alpha) * dt)
  c = 0.0 if sigma == 0 else sigma * (b - 1.0) / (sigma * kappa + kappa * kappa * alpha)
  return tuple(float(np.float32(v)) for v in (1.0 / kappa, b, c))


def stretch(omega, dt, kappa, sigma, alpha, pml_widths):
  """Per-frequency z-stretch S_E (ww, 3, Z) of the discrete CPML on the E
  components: 1/s = ik + c / (1 - b exp(-i w dt)) with E-column (integer z)
  coefficients for Ex, Ey and H-column (half-integer z) ones for Ez; cells
  outside the PML slabs have c = 0.  A^T = S_E A S_E^-1 for this operator, so
  the reciprocal adjoint is S_E A^-1 S_E^-1 r.  Where 1/s = 0 (kappa = inf,
  z-layers decoupled) the operator has no z coupling and S_E = 1."""
  Z = kappa.shape[0]
  lo, hi = pml_widths
  out = np.ones((len(omega), 3, Z), complex)
  for z in range(Z):
    inslab = z < lo or z >= Z - hi
    for col, comps in ((0, (0, 1)), (1, (2,))):
      ik, b, c = _pml_coeff(float(kappa[z, col]), float(sigma[z, col]),
                            float(alpha[z, col]), dt)
      if not inslab:
        c = 0.0
      inv = ik + c / (1 - b * np.exp(-1j * np.asarray(omega) * dt))
      for k in comps:
        out[:, k, z] = np.where(inv == 0, 1.0, 1.0 / np.where(inv == 0, 1.0, inv))
  return out


def _extend_index(n, off, size):
  return np.clip(np.arange(n) - off, 0, size - 1)


def field_and_gradient(eps, src, omega, pos, sim_params, cotangent, zz,
                       precision="f64", with_gradient=True):
  """Returns (F (ww,3,region) complex, dL/d-eps (3,region)) for the loss
  with ``dL = Re(sum conj(cotangent) dF)`` (gradient None unless asked)."""
  kw, om = pjz_ref.field_setup(eps, src, omega, pos, sim_params, zz=zz)
  dt = kw["dt"]
  mask = kw["absorption_mask"]
  X, Y = mask.shape[1:]
  Z = zz
  offset = kw["offset"]
  region = np.asarray(eps).shape[1:]
  ix = [_extend_index(n, o, s) for n, o, s in zip((X, Y, Z), offset, region)]
  eps_dom = np.asarray(eps, np.float64)[:, ix[0]][:, :, ix[1]][:, :, :, ix[2]]
  eps_dom = eps_dom.astype(np.float32)
  org, shp, prof = oracle.plane_source_box(kw["source_field"],
                                           kw["source_position"], (X, Y, Z))
  wp = pjz_ref.projection_weights(om, kw["output_steps"], dt)
  W = len(om)
  tt = kw["source_waveform"].shape[0]
  base = dict(offset=(0, 0, 0), mask=mask, kappa=kw["pml_kappa"],
              sigma=kw["pml_sigma"], alpha=kw["pml_alpha"], dt=dt, tt=tt,
              pml_widths=kw["pml_widths"], output_steps=kw["output_steps"],
              precision=precision)
  r = oracle.run(eps=eps_dom, source_origin=org, source_profile=prof,
                 waveform=kw["source_waveform"], mode="project", weights=wp,
                 **base)["out"]
  F = r[:W] + 1j * r[W:]
  sl = tuple(slice(o, o + s) for o, s in zip(offset, region))
  if not with_gradient:
    return F[(slice(None), slice(None)) + sl], None
  g = np.zeros((W, 3, X, Y, Z), complex)
  g[(slice(None), slice(None)) + sl] = cotangent

  wt = (2 / dt) * np.sin(om * dt / 2)
  # Adjoint current J = i exp(1.5 i w dt) conj(g) / w~ over g's support.
  nz = np.argwhere(np.any(g != 0, axis=(0, 1)))
  lo, hi = nz.min(axis=0), nz.max(axis=0) + 1
  bsl = tuple(slice(a, b) for a, b in zip(lo, hi))
  S = stretch(om, dt, kw["pml_kappa"], kw["pml_sigma"], kw["pml_alpha"],
              kw["pml_widths"])[:, :, None, None, :]  # (ww, 3, 1, 1, Z)
  jb = (1j * np.exp(1.5j * om * dt) / wt)[:, None, None, None, None] * (
      np.conj(g) / S)[(slice(None), slice(None)) + bsl]
  aprof = np.concatenate([jb.real, jb.imag], axis=0)
  n = np.arange(tt)
  rr = (1 + np.tanh(om[:, None] * dt * n / sim_params.source_ramp
                    - sim_params.source_delay)) / 2
  th = om[:, None] * dt * n
  awave = np.concatenate([rr * np.cos(th), -rr * np.sin(th)], axis=0).T

  # Q = w~^2 exp(-2 i w dt) F, plus i w~ exp(-1.5 i w dt) J_src / eps on the
  # cells of the source, whose profile pjz divides by epsilon.
  Q = (wt**2 * np.exp(-2j * om * dt))[:, None, None, None, None] * F
  idx = np.arange(*kw["output_steps"])
  wave = np.asarray(kw["source_waveform"], np.float64)
  samples = np.where(idx[:, None] >= 0, wave[np.clip(idx, 0, None)], 0.0)
  ph = wp @ samples
  wph = (ph[:W] + 1j * ph[W:]).T  # (ncols, ww)
  jsrc = np.einsum("kcxyz,kw->wcxyz", prof.astype(np.float64), wph)
  ssl = tuple(slice(o, o + s) for o, s in zip(org, shp))
  Q[(slice(None), slice(None)) + ssl] += (
      (1j * wt * np.exp(-1.5j * om * dt))[:, None, None, None, None] * jsrc
      / eps_dom[(slice(None),) + ssl])
  Q = Q * S
  q = np.concatenate([Q.real, Q.imag], axis=0)
  u = np.concatenate([wp[:W], -wp[W:]], axis=0)
  grad = oracle.run(eps=eps_dom, source_origin=tuple(lo), source_profile=aprof,
                    waveform=awave, mode="grad", weights=u, q=q,
                    grad_origin=(0, 0, 0), **base)["out"]
  # Fold edge-extended cells back onto the region voxel they copy.
  out = np.zeros((3,) + tuple(region))
  np.add.at(out, (slice(None),) + np.ix_(ix[0], ix[1], ix[2]), grad)
  return F[(slice(None), slice(None)) + sl], out
