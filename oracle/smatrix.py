"""FP64 restatement of the batched S-matrix gradient (test infrastructure).

Restates, on the CPU oracle engine, the n-forward + n-unit-adjoint method
the product uses for ``L = sum_w sum_ij m_ij |S_ij|^2`` (the objective of
the multi-port config; pjz's own ``scatter`` loops over ports at
``src/pjz/_field.py:354-356``).  Port geometry comes from the problem
description (plain data); profiles, sources, stretch and contraction are
written out here again.  Only ``tests/`` import it.
"""

import numpy as np

import oracle
from oracle import pjz_ref
from oracle.adjoint import stretch as cpml_stretch


def _port_profile(P, port):
  Z = P.eps.shape[3]
  t = np.arange(-P.window, P.window)[:, None] + 0.5 * (port.axis == 0)
  z = np.arange(Z)[None, :] - P.zc
  return np.exp(-(t**2 + z**2) / (2 * 7.5**2))


def _monitor(P, port):
  Z = P.eps.shape[3]
  if port.axis == 0:
    return (port.monitor, port.center - P.window, 0), (1, 2 * P.window, Z)
  return (port.center - P.window, port.monitor, 0), (2 * P.window, 1, Z)


def _comp(port):
  return 1 if port.axis == 0 else 0


def solve(P, precision="f64", eps=None, with_gradient=True, nthreads=0):
  """Returns (S (n, n, ww), L, dL/d-eps over the design box (3, box))."""
  eps = P.eps if eps is None else eps
  X, Y, Z = eps.shape[1:]
  dt = 0.5
  om = np.asarray(P.omega, np.float64)
  ww = len(om)
  it = pjz_ref.sampling_interval(om.min(), om.max(), ww, dt)
  steps = pjz_ref.output_steps(P.tt, it, ww)
  wp = pjz_ref.projection_weights(om, steps, dt)
  n_t = np.arange(P.tt)
  width, delay = P.ramp
  r = (1 + np.tanh(om[:, None] * dt * n_t / width - delay)) / 2
  rsin = np.mean(r * np.exp(1j * om[:, None] * dt * n_t), axis=0)
  fwave = np.stack([np.imag(rsin), np.zeros(P.tt)], axis=1)
  th = om[:, None] * dt * n_t
  awave = np.concatenate([r * np.cos(th), -r * np.sin(th)], axis=0).T
  kap = np.ones_like(P.pml_sigma)
  alp = np.zeros_like(P.pml_sigma)
  base = dict(offset=(0, 0, 0), mask=P.mask, kappa=kap, sigma=P.pml_sigma,
              alpha=alp, dt=dt, tt=P.tt, pml_widths=(P.pml, P.pml),
              output_steps=steps, mode="project", weights=wp,
              precision=precision, nthreads=nthreads)
  (bx, by, bz), (nx, ny, nz) = P.design_box
  dsl = (slice(None), slice(None), slice(bx, bx + nx), slice(by, by + ny),
         slice(bz, bz + nz))
  n = len(P.ports)

  def phasors(org, prof, wave):
    o = oracle.run(eps=eps, source_origin=org, source_profile=prof,
                   waveform=wave, **base)["out"]
    return o[:ww] + 1j * o[ww:]

  S = np.zeros((n, n, ww), complex)
  F = []
  for i, port in enumerate(P.ports):
    shape = (2, Y, Z) if port.axis == 0 else (X, 2, Z)
    prof = np.zeros((2, 3) + shape)
    t0 = port.center - P.window
    if port.axis == 0:
      prof[0, _comp(port), 1, t0:t0 + 2 * P.window] = _port_profile(P, port)
      org = (port.source - 1, 0, 0)
    else:
      prof[0, _comp(port), t0:t0 + 2 * P.window, 1] = _port_profile(P, port)
      org = (0, port.source - 1, 0)
    Fi = phasors(org, prof, fwave)
    for j, pj in enumerate(P.ports):
      (mo, ms) = _monitor(P, pj)
      e = Fi[:, _comp(pj), mo[0]:mo[0] + ms[0], mo[1]:mo[1] + ms[1],
             mo[2]:mo[2] + ms[2]]
      S[i, j] = np.sum(e * _port_profile(P, pj).reshape(ms), axis=(-3, -2, -1))
    F.append(Fi[dsl])
  L = float(np.sum(P.target[:, :, None] * np.abs(S) ** 2))
  if not with_gradient:
    return S, L, None
  wt = (2 / dt) * np.sin(om * dt / 2)
  coef = 1j * np.exp(1.5j * om * dt) / wt
  st = cpml_stretch(om, dt, kap, P.pml_sigma, alp, (P.pml, P.pml))
  G = []
  for port in P.ports:
    (mo, ms) = _monitor(P, port)
    j = coef[:, None, None, None] * _port_profile(P, port).reshape(ms)[None] / (
        st[:, _comp(port), None, None, :])
    prof = np.zeros((2 * ww, 3) + ms)
    prof[:ww, _comp(port)] = j.real
    prof[ww:, _comp(port)] = j.imag
    G.append(phasors(mo, prof, awave)[dsl])
  c = np.conj(2 * P.target[:, :, None] * S)
  q = wt**2 * np.exp(-2j * om * dt)
  grad = np.zeros((3, nx, ny, nz))
  for i in range(n):
    lam = sum(c[i, j][:, None, None, None, None] * G[j] for j in range(n))
    grad += np.real(np.einsum("w,wcxyz->cxyz", q, F[i] * lam))
  return S, L, grad
