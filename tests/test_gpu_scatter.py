"""pjz's ``scatter`` on the engine: values against pjz's overlap math on
bit-exact oracle fields, and the gradient of sum |S|^2 against a
directional central difference."""

import numpy as np
import pytest
import torch

import oracle
from oracle import pjz_ref
import pjz_gb300
from pjz_gb300._fdtdz import LaunchParams

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _problem():
  rng = np.random.default_rng(11)
  xx, yy, zz = 24, 18, 8
  eps = np.full((3, xx, yy, zz), 2.1, np.float32)
  eps[:, :, 6:12, 2:6] = 6.0
  eps[:, 9:14, 6:12, 2:6] = rng.uniform(2.1, 9.0, (3, 5, 6, 4)).astype(np.float32)
  omega = np.array([2 * np.pi / 20, 2 * np.pi / 18])
  y = np.arange(yy)[:, None] - 8.5
  z = np.arange(zz)[None, :] - 3.5
  prof = np.exp(-(y**2 + z**2) / 8.0)
  modes = []
  for k in range(2):
    m = np.zeros((2, 2, 1, yy, zz), complex)
    m[:, 0, 0] = prof * (1 + 0.2j * k)
    modes.append(m.astype(np.complex64))
  betas = [np.array([0.31, 0.34]), np.array([0.30, 0.33])]
  pos, is_fwd = (3, 18), (True, True)
  sp = pjz_gb300.SimParams(omega_range=(omega.min(), omega.max()), tt=4000,
                           source_ramp=float(omega.mean() * 0.5 * 150),
                           source_delay=3.0, absorption_padding=10,
                           absorption_coeff=3e-3, pml_widths=(3, 3),
                           use_reduced_precision=False,
                           launch_params=LaunchParams(zz=16))
  return eps, omega, modes, betas, pos, is_fwd, sp


def _oracle_fields(eps, src, omega, pos, sp):
  kw, om = pjz_ref.field_setup(eps, src, omega, pos, pjz_ref.SimParams(*sp[:-1]),
                               zz=16)
  domain = kw["absorption_mask"].shape[1:] + (16,)
  org, shp, prof = oracle.plane_source_box(kw["source_field"],
                                           kw["source_position"], domain)
  w = pjz_ref.projection_weights(om, kw["output_steps"], kw["dt"])
  r = oracle.run(eps=kw["epsilon"], offset=kw["offset"], mask=kw["absorption_mask"],
                 kappa=kw["pml_kappa"], sigma=kw["pml_sigma"],
                 alpha=kw["pml_alpha"], dt=kw["dt"], tt=sp.tt,
                 pml_widths=kw["pml_widths"], source_origin=org,
                 source_profile=prof, waveform=kw["source_waveform"],
                 output_steps=kw["output_steps"], mode="project", weights=w)["out"]
  ww = len(om)
  return (r[:ww] + 1j * r[ww:]).astype(np.complex64)


def test_scatter_values_match_pjz_overlap_on_oracle_fields(native):
  eps, omega, modes, betas, pos, is_fwd, sp = _problem()
  sv = pjz_gb300.scatter(torch.as_tensor(eps, device=DEV), omega,
                         [torch.as_tensor(m) for m in modes], betas, pos, is_fwd, sp)
  for i, (m, p) in enumerate(zip(modes, pos)):
    F = _oracle_fields(eps, np.mean(m, axis=0), omega, p, sp)
    a = pjz_ref.overlap(modes[i], betas[i], p, is_fwd[i], F)[:, 0]
    for j in range(len(modes)):
      want = pjz_ref.overlap(modes[j], betas[j], pos[j], is_fwd[j], F)[:, 1] / a
      np.testing.assert_allclose(sv[i][j].cpu().numpy(), want, rtol=1e-5, atol=1e-9)


def test_scatter_gradient_vs_directional_difference(native):
  eps, omega, modes, betas, pos, is_fwd, sp = _problem()
  tm = [torch.as_tensor(m) for m in modes]

  def loss(e):
    sv = pjz_gb300.scatter(e, omega, tm, betas, pos, is_fwd, sp)
    return sum((s.abs() ** 2).sum() for row in sv for s in row)

  e = torch.tensor(eps, device=DEV, requires_grad=True)
  loss(e).backward()
  g = e.grad.cpu().numpy()
  v = np.zeros_like(eps)
  v[:, 9:14, 6:12, 2:6] = np.random.default_rng(12).choice([-1.0, 1.0], (3, 5, 6, 4))
  d = 1e-2
  with torch.no_grad():
    fd = (loss(torch.as_tensor(eps + d * v, device=DEV)).item()
          - loss(torch.as_tensor(eps - d * v, device=DEV)).item()) / (2 * d)
  ad = float((g * v).sum())
  print(f"scatter directional derivative: fd {fd:.6e} adjoint {ad:.6e}")
  assert abs(fd - ad) / abs(fd) < 2e-3
