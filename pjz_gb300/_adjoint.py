"""Adjoint (reciprocity) gradients of the time-harmonic fields w.r.t. epsilon.

pjz differentiates ``scatter`` with a reciprocity VJP that keeps
``n^2 x (ww,3,xx,yy,zz)`` residual products (``src/pjz/_field.py:378-398``).
Here the gradient of any real loss of ``field``'s output comes from one
adjoint solve on the same engine, with the dL/d-eps accumulation fused into
the adjoint's sampling steps, so no time history and no residuals are kept.

Discrete derivation (units eps0 = mu0 = 1, dx = 1).  With the update
``E^{n+1} = E^n + cb (curl H^{n+1/2} - J^n - sigma E^n)`` and
``H^{n+1/2} = H^{n-1/2} - dt curl E^n``, a steady state
``E^n = Re(E^ exp(i w n dt))`` obeys ``A E^ = -i w~ exp(-i w dt/2) J^`` with
``A = curl curl - w~^2 eps + i w~ cos(w dt/2) sigma`` and the discrete
frequency ``w~ = (2/dt) sin(w dt/2)``.  The engine records E after the
update of step n and projects with phases ``w dt n``, so the returned phasor
is ``F = E^ exp(i w dt)``.  For a real loss with torch gradient ``g = dL/dF``
(``dL = Re(sum conj(g) dF)``) and a reciprocal ``A``:

  * adjoint source  ``J^_adj = i exp(3 i w dt/2) conj(g) / w~`` gives an
    adjoint phasor ``G = lambda exp(i w dt)`` with ``A lambda = exp(i w dt)
    conj(g)``;
  * ``dL/d eps_k = sum_w Re(Q_k G_k)`` with ``Q = w~^2 exp(-2 i w dt) F``;
  * a source profile that was divided by epsilon (pjz's ``_source``,
    ``src/pjz/_field.py:166-167``) adds ``Q += i w~ exp(-3 i w dt/2) J^/eps``
    on the source cells.

The z-CPML makes the operator non-reciprocal; for z-only stretching on the
Yee grid ``A^T = S A S^-1`` with ``S = diag(s_e(z)`` on Ex, Ey, ``s_h(z+1/2)``
on Ez``)`` and the discrete stretch ``1/s = ik + c / (1 - b exp(-i w dt))``
of the recursive convolution (``ik, b, c`` of the PML column).  Hence the
adjoint is ``S A^-1 S^-1 r``: the adjoint source is divided by ``S`` and ``Q``
is multiplied by ``S`` (both are 1 outside the PML slabs).

The engine's GRADIENT mode accumulates ``sum_j E_adj(t_j) (u_j . q)`` with
``u_j = [Wp[:ww, j], -Wp[ww:, j]]`` and ``q = [Re Q; Im Q]``, which equals
``sum_w Re(Q G)`` because ``G = sum_j (Wp[w, j] + i Wp[ww + w, j]) E_j``.
The adjoint source ramps in like pjz's waveform, per frequency.
"""

from typing import Sequence, Tuple

import numpy as np
import torch

from . import engine


def discrete_omega(omega, dt):
  """``w~ = (2/dt) sin(w dt / 2)``, the Yee scheme's effective frequency."""
  return (2.0 / dt) * np.sin(np.asarray(omega, np.float64) * dt / 2.0)


def _pml_coeff(kappa, sigma, alpha, dt):
  """(ik, b, c) of one CPML column entry, rounded to float32 like the engine."""
  if np.isinf(kappa):
    return 0.0, float(np.float32(np.exp(-alpha * dt))), 0.0
  b = np.exp(-(sigma / kappa + alpha) * dt)
  c = 0.0 if sigma == 0 else sigma * (b - 1.0) / (sigma * kappa + kappa * kappa * alpha)
  return tuple(float(np.float32(v)) for v in (1.0 / kappa, b, c))


def cpml_stretch(omega, dt, pml_kappa, pml_sigma, pml_alpha, pml_widths):
  """``S (ww, 3, zz)`` complex: the discrete z-stretch seen by Ex, Ey
  (integer z, column 0) and Ez (half-integer z, column 1).  Outside the PML
  slabs only kappa acts; where ``1/s = 0`` (kappa = inf, z-layers decoupled)
  the operator has no z coupling and ``S = 1``."""
  kap = np.asarray(pml_kappa, np.float64)
  sig = np.asarray(pml_sigma, np.float64)
  alp = np.asarray(pml_alpha, np.float64)
  om = np.asarray(omega, np.float64)
  Z = kap.shape[0]
  lo, hi = pml_widths
  out = np.ones((om.shape[0], 3, Z), complex)
  for z in range(Z):
    slab = z < lo or z >= Z - hi
    for col, comps in ((0, (0, 1)), (1, (2,))):
      ik, b, c = _pml_coeff(kap[z, col], sig[z, col], alp[z, col], dt)
      inv = ik + (c / (1 - b * np.exp(-1j * om * dt)) if slab else 0.0)
      s = np.where(inv == 0, 1.0, 1.0 / np.where(inv == 0, 1.0, inv))
      for k in comps:
        out[:, k, z] = s
  return out


def ramp(omega, dt, tt, width, delay):
  """Per-frequency ramp ``(1 + tanh(w dt n / width - delay)) / 2`` of pjz's
  ``_ramped_sin`` (``src/pjz/_field.py:109-113``): ``(ww, tt)``."""
  t = np.asarray(omega, np.float64)[:, None] * dt * np.arange(tt)
  return (1 + np.tanh(t / width - delay)) / 2


def adjoint_waveform(omega, dt, tt, width, delay):
  """``(tt, 2 ww)`` columns ``[r cos(w dt n) ..., -r sin(w dt n) ...]`` so that
  a profile pair ``[Re J^; Im J^]`` drives ``r Re(J^ exp(i w dt n))``."""
  om = np.asarray(omega, np.float64)
  r = ramp(om, dt, tt, width, delay)
  th = om[:, None] * dt * np.arange(tt)
  return np.concatenate([r * np.cos(th), -r * np.sin(th)], axis=0).T


def waveform_phasors(waveform, steps, omega, dt, weights):
  """Steady-state phasor of each waveform column at each frequency,
  projected exactly like the field samples: ``(ncols, ww)`` complex."""
  wave = np.asarray(waveform, np.float64)
  idx = np.arange(*steps)
  samples = np.where(idx[:, None] >= 0, wave[np.clip(idx, 0, None)], 0.0)
  out = np.asarray(weights, np.float64) @ samples  # (2ww, ncols)
  ww = len(omega)
  return (out[:ww] + 1j * out[ww:]).T


def nonzero_box(g: torch.Tensor) -> Tuple[Tuple[int, int, int], Tuple[int, int, int]]:
  """Bounding box (origin, shape) of the nonzero cells of ``g (..., X, Y, Z)``."""
  nz = (g != 0).reshape(-1, *g.shape[-3:]).any(dim=0)
  if not bool(nz.any()):
    return (0, 0, 0), (1, 1, 1)
  lo, hi = [], []
  for ax in range(3):
    other = tuple(a for a in range(3) if a != ax)
    hit = torch.nonzero(nz.any(dim=other)).flatten()
    lo.append(int(hit[0]))
    hi.append(int(hit[-1]) + 1)
  return tuple(lo), tuple(h - l for l, h in zip(lo, hi))


def adjoint_source(g: torch.Tensor, omega, dt, origin, shape, stretch=None):
  """Profile ``(2 ww, 3, box)`` float32 of the adjoint current for cotangent
  ``g (ww, 3, X, Y, Z)`` (complex, domain frame) inside the box; ``stretch``
  ``(ww, 3, Z)`` divides it (the ``S^-1 r`` of the CPML adjoint)."""
  om = np.asarray(omega, np.float64)
  wt = discrete_omega(om, dt)
  coef = 1j * np.exp(1.5j * om * dt) / wt  # (ww,)
  sl = tuple(slice(o, o + s) for o, s in zip(origin, shape))
  gb = g[(slice(None), slice(None)) + sl].to(torch.complex128)
  c = torch.as_tensor(coef, dtype=torch.complex128, device=g.device)
  j = c[:, None, None, None, None] * torch.conj(gb)
  if stretch is not None:
    s = torch.as_tensor(stretch, dtype=torch.complex128, device=g.device)
    j = j / s[:, :, None, None, sl[2]]
  return torch.cat([j.real, j.imag], dim=0).to(torch.float32).contiguous()


def gradient_q(F: torch.Tensor, omega, dt, src_term=None, stretch=None):
  """``q = [Re Q; Im Q]`` ``(2 ww, 3, X, Y, Z)`` float32 with
  ``Q = S (w~^2 exp(-2 i w dt) F (+ src_term))``."""
  om = np.asarray(omega, np.float64)
  wt = discrete_omega(om, dt)
  c = torch.as_tensor(wt**2 * np.exp(-2j * om * dt), dtype=torch.complex64,
                      device=F.device)
  Q = c[:, None, None, None, None] * F.to(torch.complex64)
  if src_term is not None:
    Q = Q + src_term
  if stretch is not None:
    s = torch.as_tensor(stretch, dtype=torch.complex64, device=F.device)
    Q = Q * s[:, :, None, None, :]
  return torch.cat([Q.real, Q.imag], dim=0).to(torch.float32).contiguous()


def gradient_weights(weights):
  """Sample weights ``u = [Wp[:ww]; -Wp[ww:]]`` of the GRADIENT mode."""
  w = np.asarray(weights, np.float64)
  ww = w.shape[0] // 2
  return np.concatenate([w[:ww], -w[ww:]], axis=0)


def run_adjoint(*, g: torch.Tensor, F: torch.Tensor, omega, dt, tt,
                ramp_width, ramp_delay, weights, output_steps, epsilon_domain,
                absorption_mask, pml_widths, pml_kappa, pml_sigma, pml_alpha,
                src_term=None, launch=None) -> torch.Tensor:
  """One fused adjoint solve over the whole domain; returns dL/d-eps
  ``(3, X, Y, Z)`` for every cell of ``epsilon_domain (3, X, Y, Z)``."""
  X, Y, Z = (int(v) for v in epsilon_domain.shape[1:])
  stretch = cpml_stretch(omega, dt, pml_kappa, pml_sigma, pml_alpha, pml_widths)
  origin, shape = nonzero_box(g)
  prof = adjoint_source(g, omega, dt, origin, shape, stretch)
  wave = torch.as_tensor(adjoint_waveform(omega, dt, tt, ramp_width, ramp_delay),
                         dtype=torch.float32, device=g.device)
  q = gradient_q(F, omega, dt, src_term, stretch)
  u = gradient_weights(weights)
  knobs = launch or {}
  plan = engine.Plan(
      domain=(X, Y, Z), offset=(0, 0, 0), region=(X, Y, Z), tt=tt, dt=dt,
      pml_widths=pml_widths, pml_kappa=pml_kappa, pml_sigma=pml_sigma,
      pml_alpha=pml_alpha, source_origin=origin, source_shape=shape,
      source_ncols=prof.shape[0], output_steps=output_steps,
      out_mode=engine.OUT_GRADIENT, weights=u, grad_origin=(0, 0, 0),
      grad_shape=(X, Y, Z), **knobs)
  grad, _ = plan.run(epsilon=epsilon_domain, absorption_mask=absorption_mask,
                     source=prof, waveform=wave, q=q)
  return grad


def extend_epsilon(eps: torch.Tensor, domain: Sequence[int], offset) -> torch.Tensor:
  """Edge-extends the epsilon region onto the whole domain (what the engine
  does for cells outside the region): ``(3, X, Y, Z)``."""
  idx = [torch.clamp(torch.arange(n, device=eps.device) - o, 0, s - 1)
         for n, o, s in zip(domain, offset, eps.shape[1:])]
  return eps[:, idx[0]][:, :, idx[1]][:, :, :, idx[2]].contiguous()


def fold_to_region(grad: torch.Tensor, region, offset) -> torch.Tensor:
  """Adjoint of :func:`extend_epsilon`: sums domain gradients onto the
  region cell each domain cell copies.  Along each axis the cells below the
  region fold onto its first cell and those above onto its last; the sums
  are plain reductions (no atomics), so the result is deterministic."""
  out = grad
  for ax, (o, s) in enumerate(zip(offset, region)):
    d = ax + 1
    n = out.shape[d]
    mid = out.narrow(d, o, s).clone()
    if o > 0:
      mid.narrow(d, 0, 1).add_(out.narrow(d, 0, o).sum(dim=d, keepdim=True))
    if o + s < n:
      mid.narrow(d, s - 1, 1).add_(
          out.narrow(d, o + s, n - o - s).sum(dim=d, keepdim=True))
    out = mid
  return out
