"""Batched S-matrix (n forwards + n unit adjoints in one launch): equal to
the serial loop of the same solves, equal to the same method in FP64 on the
CPU oracle, whose gradient matches FP64 central differences.

Finite differences of the FP32 forward are not used here: the objective of
this geometry is ~600 (unnormalised overlaps next to the sources), so its
FP32 rounding noise (~1e-7 relative) swamps differences at delta-eps 1e-3.
"""

import numpy as np
import pytest
import torch

from oracle import smatrix as osm
from pjz_gb300 import smatrix

pytestmark = pytest.mark.gpu


def _small(tt=9000, **kw):
  # Three frequencies 20 nm apart sample over 5928 steps (interval 988), so
  # the window must start after the (100-step) ramp has settled.
  return smatrix.build_c4(domain=(256, 256, 32), tt=tt, device_cells=40, edge=24,
                          monitor_inset=12, window=16, pml=4, ramp_steps=100,
                          **kw)


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


def _tiny():
  return smatrix.build_c4(domain=(80, 80, 16), tt=9000, device_cells=16, edge=10,
                          monitor_inset=6, window=8, pml=3, ramp_steps=100)


def test_smatrix_matches_fp64_oracle_and_finite_differences(native):
  """GPU batched S, objective and gradient against the same method restated
  in FP64 on the CPU oracle; the FP64 gradient against FP64 central
  differences (delta-eps 1e-3) at design voxels."""
  P = _tiny()
  s = smatrix.SMatrixSolver(P)
  s.run_batched()
  S, L, grad = s.results()
  S64, L64, g64 = osm.solve(P)
  errS = np.linalg.norm(S.cpu().numpy() - S64) / np.linalg.norm(S64)
  errg = np.linalg.norm(grad.cpu().numpy() - g64) / np.linalg.norm(g64)
  print(f"S-matrix GPU vs FP64: S {errS:.2e}, L {abs(L.item() - L64) / L64:.2e}, "
        f"grad {errg:.2e}")
  assert errS < 1e-4 and errg < 1e-4
  (bx, by, bz), _ = P.design_box
  pts = [(1, 5, 7, 2), (0, 9, 3, 3), (1, 12, 12, 1)]
  fd, ad = [], []
  for p in pts:
    d = 1e-3
    q = (p[0], bx + p[1], by + p[2], bz + p[3])
    ep, em = P.eps.copy(), P.eps.copy()
    ep[q] += d
    em[q] -= d
    Lp = osm.solve(P, eps=ep, with_gradient=False)[1]
    Lm = osm.solve(P, eps=em, with_gradient=False)[1]
    fd.append((Lp - Lm) / (2 * d))
    ad.append(g64[p])
  fd, ad = np.array(fd), np.array(ad)
  err = np.linalg.norm(fd - ad) / np.linalg.norm(fd)
  print("FP64 S-matrix gradient vs FD:", err, fd, ad)
  assert err < 1e-3


def test_device_assembly_matches_torch_restatement(native):
  """S, objective and gradient from the device kernels (plane overlaps and
  the FP64 gradient product) against the same sums written as complex128
  torch reductions over the same recorded phasors."""
  import numpy as _np
  from pjz_gb300 import _adjoint
  P = _tiny()
  s = smatrix.SMatrixSolver(P)
  s.run_batched()
  S, L, grad = s.results()
  n, ww = len(P.ports), len(P.omega)
  cplx = lambda a: torch.complex(a[:ww], a[ww:])
  Sref = torch.zeros((n, n, ww), dtype=torch.complex128, device=S.device)
  F = []
  for i in range(n):
    views = s.plans[i].split(s.outs[i])
    F.append(cplx(views[0]).to(torch.complex128))
    for j, port in enumerate(P.ports):
      e = cplx(views[1 + j])[:, smatrix._transverse(port)].to(torch.complex128)
      p = torch.as_tensor(smatrix._port_profile(P, port), device=S.device,
                          dtype=torch.float64).reshape(e.shape[1:])
      Sref[i, j] = (e * p).sum(dim=(-3, -2, -1))
  G = torch.stack([cplx(s.plans[n + j].split(s.outs[n + j])[0]) for j in range(n)]
                  ).to(torch.complex128)
  m = torch.as_tensor(P.target, device=S.device, dtype=torch.float64)
  Lref = (m[:, :, None] * Sref.abs() ** 2).sum()
  c = torch.conj(2 * m[:, :, None] * Sref)
  wt = _adjoint.discrete_omega(P.omega, 0.5)
  q = torch.as_tensor(wt**2 * _np.exp(-2j * P.omega * 0.5), device=S.device,
                      dtype=torch.complex128)
  cg = torch.einsum("ijw,jwcxyz->iwcxyz", c, G)
  gref = torch.einsum("w,iwcxyz->cxyz", q, torch.stack(F) * cg).real
  torch.testing.assert_close(S, Sref, rtol=1e-12, atol=0)
  assert abs(float(L) - float(Lref)) <= 1e-12 * float(Lref)
  # coefficients pass as float32 into the kernel; FP64 sums otherwise
  torch.testing.assert_close(grad.double(), gref, rtol=1e-5, atol=1e-6 * float(gref.abs().max()))
