"""Batched S-matrix (n forwards + n unit adjoints in one launch): equal to
the serial loop of the same solves, and its epsilon-gradient against a
directional central difference of the objective."""

import numpy as np
import pytest
import torch

from pjz_gb300 import smatrix

pytestmark = pytest.mark.gpu


def _small(tt=6000, **kw):
  return smatrix.build_c4(domain=(256, 256, 32), tt=tt, device_cells=40, edge=24,
                          monitor_inset=12, window=16, pml=4, **kw)


def test_batched_equals_serial(native):
  s = smatrix.SMatrixSolver(_small(tt=800))
  s.run_serial()
  torch.cuda.synchronize()
  ref = [o.clone() for o in s.outs]
  for _ in range(2):  # capture, then replay
    for o in s.outs:
      o.fill_(float("nan"))
    s.run_batched(graph=True)
    torch.cuda.synchronize()
    for a, b in zip(s.outs, ref):
      assert torch.equal(a, b)
  s.batch.check_status()


def test_smatrix_gradient_vs_directional_difference(native):
  P = _small()
  s = smatrix.SMatrixSolver(P)
  s.run_batched()
  S, L, grad = s.results()
  assert torch.isfinite(S).all() and L.item() > 0
  (bx, by, bz), (nx, ny, nz) = P.design_box
  rng = np.random.default_rng(7)
  v = np.zeros_like(P.eps)
  v[:, bx:bx + nx, by:by + ny, bz:bz + nz] = rng.choice([-1.0, 1.0], (3, nx, ny, nz))

  def L_of(eps):
    q = smatrix.SMatrixSolver(P._replace(eps=eps.astype(np.float32)))
    q.run_batched(graph=False)
    return q.results()[1].item()

  d = 1e-2
  fd = (L_of(P.eps + d * v) - L_of(P.eps - d * v)) / (2 * d)
  ad = float((grad.cpu().numpy() * v[:, bx:bx + nx, by:by + ny, bz:bz + nz]).sum())
  err = abs(fd - ad) / abs(fd)
  print(f"S-matrix directional derivative: fd {fd:.6e} adjoint {ad:.6e} rel {err:.2e}")
  assert err < 2e-3
