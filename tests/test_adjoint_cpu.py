"""Adjoint method checked on the CPU: the package's adjoint helpers
(``pjz_gb300/_adjoint.py``) driven through the FP64 oracle, against central
finite differences of the same FP64 forward solve."""

import numpy as np
import pytest
import torch

import oracle
from oracle import pjz_ref
from pjz_gb300 import _adjoint


def _problem():
  X, Y, Z, tt, dt = 32, 28, 16, 3200, 0.5
  omega = np.array([2 * np.pi / 20, 2 * np.pi / 18])
  eps = np.full((3, X, Y, Z), 2.0, np.float32)
  eps[:, 8:24, 10:18, 6:10] = 6.0
  mask = pjz_ref.absorption_mask(X, Y, 7, 3e-3).astype(np.float32)
  sig = pjz_ref.pml_sigma((3, 3), Z, 0.5, 1.3).astype(np.float32)
  W = len(omega)
  interval = pjz_ref.sampling_interval(omega.min(), omega.max(), W, dt)
  steps = pjz_ref.output_steps(tt, interval, W)
  wp = pjz_ref.projection_weights(omega, steps, dt)
  width, delay = float(omega.mean() * dt * 150), 3.0
  r = _adjoint.ramp(omega, dt, tt, width, delay)
  n = np.arange(tt)
  rsin = np.mean(r * np.exp(1j * omega[:, None] * dt * n), axis=0)
  prof = np.zeros((1, 3, 1, Y, Z), np.float32)
  prof[0, 1, 0, 10:18, 6:10] = 1.0
  base = dict(offset=(0, 0, 0), mask=mask, kappa=np.ones_like(sig), sigma=sig,
              alpha=0.05 * np.ones_like(sig), dt=dt, pml_widths=(3, 3),
              output_steps=steps, precision="f64", tt=tt)
  return dict(X=X, Y=Y, Z=Z, tt=tt, dt=dt, omega=omega, eps=eps, W=W, wp=wp,
              steps=steps, width=width, delay=delay, prof=prof,
              wave=np.imag(rsin).astype(np.float32)[:, None], base=base)


def _forward(P, eps):
  r = oracle.run(eps=eps, source_origin=(6, 0, 0), source_profile=P["prof"],
                 waveform=P["wave"], mode="project", weights=P["wp"],
                 **P["base"])["out"]
  return r[:P["W"]] + 1j * r[P["W"]:]


def test_adjoint_gradient_matches_central_differences():
  P = _problem()
  rng = np.random.default_rng(0)
  c = np.zeros((P["W"], 3, P["X"], P["Y"], P["Z"]), complex)
  c[:, 1, 26, 9:19, 5:11] = rng.normal(size=(P["W"], 10, 6)) + 1j * rng.normal(
      size=(P["W"], 10, 6))
  loss = lambda F: np.real(np.sum(np.conj(c) * F))
  F = _forward(P, P["eps"])
  g = torch.as_tensor(c)  # L = Re(sum conj(c) F)  =>  dL/dF = c
  origin, shape = _adjoint.nonzero_box(g)
  prof = _adjoint.adjoint_source(g, P["omega"], P["dt"], origin, shape).numpy()
  wave = _adjoint.adjoint_waveform(P["omega"], P["dt"], P["tt"], P["width"],
                                   P["delay"])
  q = _adjoint.gradient_q(torch.as_tensor(F), P["omega"], P["dt"]).numpy()
  u = _adjoint.gradient_weights(P["wp"])
  grad = oracle.run(eps=P["eps"], source_origin=origin, source_profile=prof,
                    waveform=wave, mode="grad", weights=u, q=q,
                    grad_origin=(0, 0, 0), **P["base"])["out"]
  pts = [(1, 16, 14, 8), (0, 12, 12, 7), (2, 20, 15, 9), (1, 22, 11, 6),
         (1, 10, 16, 8), (0, 18, 14, 8)]
  fd, ad = [], []
  for p in pts:
    d = 1e-3
    ep, em = P["eps"].copy(), P["eps"].copy()
    ep[p] += d
    em[p] -= d
    fd.append((loss(_forward(P, ep)) - loss(_forward(P, em))) / (2 * d))
    ad.append(grad[p])
  fd, ad = np.array(fd), np.array(ad)
  err = np.linalg.norm(fd - ad) / np.linalg.norm(fd)
  assert err < 1e-3, (err, fd, ad)


def test_fold_is_adjoint_of_extend():
  rng = np.random.default_rng(1)
  eps = torch.as_tensor(rng.normal(size=(3, 4, 5, 3)))
  g = torch.as_tensor(rng.normal(size=(3, 9, 8, 7)))
  ext = _adjoint.extend_epsilon(eps, (9, 8, 7), (2, 1, 3))
  fold = _adjoint.fold_to_region(g, (4, 5, 3), (2, 1, 3))
  assert torch.allclose((ext * g).sum(), (eps * fold).sum())


def test_waveform_phasors_of_pure_tones():
  omega = np.array([0.15, 0.17])
  dt, tt = 0.5, 3000
  interval = pjz_ref.sampling_interval(0.15, 0.17, 2, dt)
  steps = pjz_ref.output_steps(tt, interval, 2)
  wp = pjz_ref.projection_weights(omega, steps, dt)
  n = np.arange(tt)
  wave = np.stack([np.sin(0.15 * dt * n), np.cos(0.17 * dt * n)], axis=1)
  ph = _adjoint.waveform_phasors(wave, steps, omega, dt, wp)
  np.testing.assert_allclose(ph, [[-1j, 0], [0, 1]], atol=1e-9)


def test_fp64_oracle_adjoint_matches_finite_differences():
  """The FP64 restatement of the field adjoint (with the CPML stretch
  correction, source-plane term and edge folding) against central
  differences on a converging geometry."""
  from oracle import adjoint as oradj
  rng = np.random.default_rng(3)
  xx, yy, zz = 22, 18, 8
  eps = np.full((3, xx, yy, zz), 2.1, np.float32)
  eps[:, 8:14, 6:12, 2:6] = 9.0
  src = np.zeros((2, 1, yy, zz), np.float32)
  src[0, 0, 6:12, 2:6] = 1.0
  omega = np.array([2 * np.pi / 20, 2 * np.pi / 18])
  sp = pjz_ref.SimParams(omega_range=(omega.min(), omega.max()), tt=3000,
                         source_ramp=float(omega.mean() * 0.5 * 150),
                         source_delay=3.0, absorption_padding=10,
                         absorption_coeff=3e-3, pml_widths=(4, 4),
                         use_reduced_precision=False)
  c = np.zeros((2, 3, xx, yy, zz), complex)
  c[:, 1, 18, 5:13, 1:7] = rng.normal(size=(2, 8, 6)) + 1j * rng.normal(size=(2, 8, 6))
  _, grad = oradj.field_and_gradient(eps, src, omega, 3, sp, c, zz=16)
  loss = lambda e: np.real(np.sum(np.conj(c) * oradj.field_and_gradient(
      e, src, omega, 3, sp, c, zz=16, with_gradient=False)[0]))
  pts = [(1, 11, 9, 4), (1, 3, 8, 3), (1, 0, 9, 3), (2, 11, 9, 7)]
  fd = []
  for p in pts:
    d = 1e-3
    ep, em = eps.copy(), eps.copy()
    ep[p] += d
    em[p] -= d
    fd.append((loss(ep) - loss(em)) / (2 * d))
  fd = np.array(fd)
  ad = np.array([grad[p] for p in pts])
  assert np.linalg.norm(fd - ad) / np.linalg.norm(fd) < 1e-3, (fd, ad)


@pytest.mark.parametrize("pml,kappa_val,alpha_val", [
    ((4, 4), 1.0, 0.05), ((3, 5), 2.0, 0.0), ((0, 6), 1.5, 0.1), ((4, 4), np.inf, 0.0)])
def test_cpml_stretch_matches_oracle(pml, kappa_val, alpha_val):
  """The product's CPML stretch (used by the S-matrix unit adjoints) equals
  the oracle's, which the time-domain reciprocity KAT pins: kappa != 1,
  alpha != 0, one-sided slabs and kappa = inf."""
  from oracle import adjoint as oadj
  from pjz_gb300 import _adjoint
  Z = 16
  sig = pjz_ref.pml_sigma(pml, Z, 0.5, 1.3)
  kap = np.full_like(sig, kappa_val)
  alp = np.full_like(sig, alpha_val)
  om = np.array([0.12, 0.16215, 0.3])
  got = _adjoint.cpml_stretch(om, 0.5, kap, sig, alp, pml)
  want = oadj.stretch(om, 0.5, kap, sig, alp, pml)
  np.testing.assert_allclose(got, want, rtol=1e-12, atol=0)


@pytest.mark.parametrize("region,offset", [((10, 9, 6), (4, 3, 2)),
                                           ((20, 17, 12), (0, 0, 0)),
                                           ((5, 17, 1), (15, 0, 11))])
def test_fold_to_region_sums_each_copied_cell(region, offset):
  """The gradient fold (adjoint of the edge extension) adds every domain
  cell onto the region cell it copies, with plain reductions: equal to an
  explicit per-cell loop, and identical on repeated calls."""
  g = torch.randn(3, 20, 17, 12, dtype=torch.float64,
                  generator=torch.Generator().manual_seed(0))
  want = np.zeros((3,) + region)
  gn = g.numpy()
  for x in range(20):
    for y in range(17):
      for z in range(12):
        r = [min(max(v - o, 0), s - 1) for v, o, s in zip((x, y, z), offset, region)]
        want[:, r[0], r[1], r[2]] += gn[:, x, y, z]
  a = _adjoint.fold_to_region(g, region, offset)
  np.testing.assert_allclose(a.numpy(), want, rtol=1e-12, atol=1e-12)
  assert torch.equal(a, _adjoint.fold_to_region(g, region, offset))
