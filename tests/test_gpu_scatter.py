"""pjz's ``scatter`` on the engine: values against pjz's overlap math on
bit-exact oracle fields, the monitor-plane path against the full-field
path bit for bit (with outputs of plane size), per-frequency sources
against per-frequency oracle solves, and the gradient of sum |S|^2 against
a directional central difference."""

import numpy as np
import pytest
import torch

import oracle
from oracle import pjz_ref
import pjz_gb300
from pjz_gb300 import _scatter, engine
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


def _full_field_svals(eps, omega, modes, betas, pos, is_fwd, sp):
  """pjz's scatter by the book: one full-field ``field`` solve per port and
  the overlap on slices of those fields; returns (svals, fields)."""
  e = torch.as_tensor(eps, device=DEV)
  tm = [torch.as_tensor(m) for m in modes]
  fields = [pjz_gb300.field(e, torch.mean(m, dim=0), omega, p, sp)
            for m, p in zip(tm, pos)]
  out = []
  for i, f in enumerate(fields):
    a = _scatter._overlap(tm[i], betas[i], pos[i], is_fwd[i], f)[:, 0]
    out.append([_scatter._overlap(tm[j], betas[j], pos[j], is_fwd[j], f)[:, 1] / a
                for j in range(len(tm))])
  return out, fields


def test_scatter_monitor_planes_equal_full_fields(native, monkeypatch):
  """Without gradients scatter records only the overlap planes, in one
  batched launch: the recorded planes equal the full fields' slices bit for
  bit, the values equal the full-field path (to the rounding of the
  overlap sums, 1e-12), and the recorded outputs are plane-sized."""
  eps, omega, modes, betas, pos, is_fwd, sp = _problem()
  want, fields = _full_field_svals(eps, omega, modes, betas, pos, is_fwd, sp)
  tm = [torch.as_tensor(m) for m in modes]
  planes = [(0, 4), (0, 5), (0, 19), (0, 20)]
  rec = _scatter._plane_phasors(torch.as_tensor(eps, device=DEV),
                                _scatter._solves(tm, pos, omega, sp, False), planes)
  for f, r in zip(fields, rec):
    for (ax, x) in planes:
      assert torch.equal(r[(ax, x)], f[:, :, x:x + 1]), x
  sizes = []
  run = engine.Batch.run

  def spy(self, inputs, graph=True):
    res = run(self, inputs, graph)
    sizes.extend(out.numel() for out, _ in res)
    return res
  monkeypatch.setattr(engine.Batch, "run", spy)
  got = pjz_gb300.scatter(torch.as_tensor(eps, device=DEV), omega,
                          [torch.as_tensor(m) for m in modes], betas, pos, is_fwd,
                          sp)
  for i in range(len(modes)):
    for j in range(len(modes)):
      torch.testing.assert_close(got[i][j], want[i][j], rtol=1e-12, atol=0)
  # Two ports x-normal, forward: planes x = 4, 5 and 19, 20, each
  # (2 ww rows, 3, 1, yy, zz) floats; the full field is (2 ww, 3, xx, yy, zz).
  ww, (_, xx, yy, zz) = len(omega), eps.shape
  assert sizes == [4 * 2 * ww * 3 * yy * zz] * 2
  assert sizes[0] * xx == 4 * (2 * ww * 3 * xx * yy * zz)  # 4 of xx planes


def test_scatter_per_frequency_sources_match_oracle(native):
  """per_frequency=True: one solve per (port, frequency) with that
  frequency's mode and a single-frequency ramp; against the same solves on
  the FP32 oracle with pjz's overlap math (bit-exact fields, so the values
  agree to the overlap's rounding), and against the engine's full-field
  single-frequency solves bit for bit."""
  eps, omega, modes, betas, pos, is_fwd, sp = _problem()
  # Modes that differ across frequency, so averaging would matter.
  modes = [m.copy() for m in modes]
  for m in modes:
    m[1] *= np.exp(0.3j) * 1.4
  sv = pjz_gb300.scatter(torch.as_tensor(eps, device=DEV), omega,
                         [torch.as_tensor(m) for m in modes], betas, pos, is_fwd,
                         sp, per_frequency=True)
  sv_avg = pjz_gb300.scatter(torch.as_tensor(eps, device=DEV), omega,
                             [torch.as_tensor(m) for m in modes], betas, pos,
                             is_fwd, sp)
  n = len(modes)
  for k in range(len(omega)):
    om = omega[k:k + 1]
    spk = sp._replace(omega_range=(float(om[0]), float(om[0])))
    mk = [m[k:k + 1] for m in modes]
    bk = [np.asarray(b)[k:k + 1] for b in betas]
    for i in range(n):
      F = _oracle_fields(eps, modes[i][k], om, pos[i], spk)
      a = pjz_ref.overlap(mk[i], bk[i], pos[i], is_fwd[i], F)[:, 0]
      ef = pjz_gb300.field(torch.as_tensor(eps, device=DEV),
                           torch.as_tensor(modes[i][k]), om, pos[i], spk)
      assert np.array_equal(ef.cpu().numpy(), F)
      for j in range(n):
        want = pjz_ref.overlap(mk[j], bk[j], pos[j], is_fwd[j], F)[:, 1] / a
        got = sv[i][j][k:k + 1].cpu().numpy()
        # Same fields; the overlap sums (complex64) differ only in order.
        np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-12)
  assert all(torch.isfinite(v).all() for row in sv_avg for v in row)
