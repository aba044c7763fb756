"""GPU adjoint: ``field``'s autograd backward (one fused adjoint solve)
against central finite differences.

* small cases: the whole gradient against the same adjoint restated in FP64
  on the CPU oracle, and FD of the FP64 oracle forward (exact arithmetic)
  at interior, region-boundary (edge-extended) and source-plane voxels;
* c2: the 512x512x64 c1 geometry, objective sum_w |port . E_y(x_out)|^2,
  FD of the GPU FP32 forward along the gradient's sign pattern (1e-3), along
  a random direction and at single voxels (1e-2, the FP32 noise floor);
  and at 16 seeded single voxels against the tangent-linear derivative
  (``pjz_gb300._tangent``: the exact directional derivative of the solve,
  with no difference taken, so FP32 noise does not swamp it), 1e-3.
Small cases: 1e-3 relative (vector norm over the checked voxels).
"""

import numpy as np
import pytest
import torch

import oracle
from oracle import adjoint as oradj
from oracle import pjz_ref
import pjz_gb300
from pjz_gb300 import _tangent, workloads
from pjz_gb300._fdtdz import LaunchParams

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _small(isolated=True, tt=4000):
  """Small pjz problem: a scatterer (isolated, or a waveguide running into
  the absorber), an x-normal source at an odd position (bumped, flipped
  columns) and a monitor cotangent on a plane."""
  rng = np.random.default_rng(3)
  xx, yy, zz = 22, 18, 8
  eps = np.full((3, xx, yy, zz), 2.1, np.float32)
  if isolated:
    eps[:, 8:14, 6:12, 2:6] = 9.0
  else:
    eps[:, :, 6:12, 2:6] = 9.0
  eps[:, 9:13, 7:11, 2:6] += rng.uniform(-1, 1, (3, 4, 4, 4)).astype(np.float32)
  src = np.zeros((2, 1, yy, zz), np.float32)
  src[0, 0, 6:12, 2:6] = 1.0
  omega = np.array([2 * np.pi / 20, 2 * np.pi / 18])
  sp = pjz_gb300.SimParams(omega_range=(omega.min(), omega.max()), tt=tt,
                           source_ramp=float(omega.mean() * 0.5 * 150),
                           source_delay=3.0, absorption_padding=10,
                           absorption_coeff=3e-3, pml_widths=(3, 3),
                           use_reduced_precision=False,
                           launch_params=LaunchParams(zz=16))
  c = np.zeros((2, 3, xx, yy, zz), complex)
  c[:, 1, 18, 5:13, 1:7] = rng.normal(size=(2, 8, 6)) + 1j * rng.normal(size=(2, 8, 6))
  return eps, src, omega, 3, sp, c


# interior, source plane (x = 3), region edges (edge-extended into the
# absorber and the z-PML).
POINTS = [(1, 11, 9, 4), (0, 10, 8, 3), (2, 12, 10, 4), (1, 3, 8, 3),
          (1, 3, 10, 4), (1, 0, 9, 3), (1, 21, 9, 4), (0, 11, 0, 3),
          (2, 11, 9, 7)]


def _gpu_grad(eps, src, omega, pos, sp, c):
  e = torch.tensor(eps, device=DEV, requires_grad=True)
  F = pjz_gb300.field(e, torch.as_tensor(src, device=DEV), omega, pos, sp)
  ct = torch.as_tensor(c, dtype=torch.complex64, device=DEV)
  torch.real(torch.sum(torch.conj(ct) * F)).backward()
  return F.detach().cpu().numpy(), e.grad.cpu().numpy()


def _oracle_sp(sp):
  return pjz_ref.SimParams(*sp[:-1])


@pytest.mark.parametrize("isolated", [True, False])
def test_field_backward_matches_fp64_oracle_adjoint(native, isolated):
  """Same adjoint method in FP64 on the CPU oracle: the whole gradient."""
  eps, src, omega, pos, sp, c = _small(isolated, tt=2500)
  _, got = _gpu_grad(eps, src, omega, pos, sp, c)
  _, want = oradj.field_and_gradient(eps, src, omega, pos, _oracle_sp(sp), c, zz=16)
  err = np.linalg.norm(got - want) / np.linalg.norm(want)
  print("GPU FP32 adjoint vs FP64 oracle adjoint: rel-L2", err)
  assert err < 1e-4


def test_field_backward_vs_fp64_finite_differences(native):
  """Converging geometry: adjoint vs central differences of the FP64
  oracle forward (delta-eps 1e-3), 1e-3 relative."""
  eps, src, omega, pos, sp, c = _small(True)
  _, grad = _gpu_grad(eps, src, omega, pos, sp, c)
  loss = lambda e: np.real(np.sum(np.conj(c) * oradj.field_and_gradient(
      e, src, omega, pos, _oracle_sp(sp), c, zz=16, with_gradient=False)[0]))
  fd = []
  for p in POINTS:
    d = 1e-3
    ep, em = eps.copy(), eps.copy()
    ep[p] += d
    em[p] -= d
    fd.append((loss(ep) - loss(em)) / (2 * d))
  fd = np.array(fd)
  ad = np.array([grad[p] for p in POINTS])
  err = np.linalg.norm(fd - ad) / np.linalg.norm(fd)
  print("small adjoint vs FP64 FD:", err, fd, ad)
  assert err < 1e-3


def test_c2_gradient_vs_finite_differences(native):
  """c2: c1 geometry (512x512x64, 5 frequencies, blurred random 50x50x6
  design region), objective sum_w |port . E_y(x_out)|^2.

  The random design region rings down slowly: the objective is 0.8% off its
  steady state at 10000 steps and settles (1e-6) by 20000, so the check runs
  20000 steps -- the adjoint returns the steady-state gradient.

  The FP32 objective (L ~ 2.2) carries about 2e-7 of rounding noise that
  changes with every perturbed input, so a central difference at step d has
  noise ~3e-7 / (2 d).  The checks are sized against that floor:
    * along v = sign(grad) on the design box the derivative is sum |grad|
      (~10, so noise below 1e-5 relative at d = 1e-3); d = 1e-3 and 2e-3 must
      agree with each other (truncation) and with the adjoint to 1e-3;
    * along a random +-1 direction (derivative ~6e-3, noise ~2e-3 relative at
      d = 1e-2) and at 8 single voxels (delta-eps 0.1, noise ~4e-3 rel-L2)
      the tolerance is 1e-2.
  """
  wl = workloads.design_c1(tt=20000)
  eps = torch.tensor(wl.epsilon, device=DEV, requires_grad=True)
  src = torch.as_tensor(wl.source, device=DEV)
  port = torch.as_tensor(workloads.port_profile(wl), device=DEV)
  F = pjz_gb300.field(eps, src, wl.omega, wl.source_pos, wl.sim_params)
  workloads.overlap_objective(F, wl, port).backward()
  grad = eps.grad.cpu().numpy()

  def L(e):
    with torch.no_grad():
      out = pjz_gb300.field(torch.as_tensor(e, device=DEV), src, wl.omega,
                            wl.source_pos, wl.sim_params)
      return workloads.overlap_objective(out, wl, port,
                                         dtype=torch.complex128).item()

  def fd_along(v, d):
    return (L(wl.epsilon + d * v) - L(wl.epsilon - d * v)) / (2 * d)

  (bx, by, bz), (nx, ny, nz) = wl.design_box
  box = (slice(None), slice(bx, bx + nx), slice(by, by + ny), slice(bz, bz + nz))

  v = np.zeros_like(wl.epsilon)
  v[box] = np.sign(grad[box])
  ad_sign = float(np.sum(grad * v))
  fd1, fd2 = fd_along(v, 1e-3), fd_along(v, 2e-3)
  err_sign = abs(fd1 - ad_sign) / abs(ad_sign)
  print(f"c2 along sign(grad): fd(1e-3) {fd1:.8e} fd(2e-3) {fd2:.8e} "
        f"adjoint {ad_sign:.8e} rel {err_sign:.2e}")

  rng = np.random.default_rng(1)
  v = np.zeros_like(wl.epsilon)
  v[box] = rng.choice([-1.0, 1.0], (3, nx, ny, nz))
  fd_dir = fd_along(v, 1e-2)
  ad_dir = float(np.sum(grad * v))
  err_dir = abs(fd_dir - ad_dir) / abs(fd_dir)
  print(f"c2 random direction: fd {fd_dir:.6e} adjoint {ad_dir:.6e} rel {err_dir:.2e}")

  pts = [(1, bx + int(rng.integers(nx)), by + int(rng.integers(ny)),
          bz + int(rng.integers(nz))) for _ in range(8)]
  fd, ad = [], []
  for p in pts:
    ep, em = wl.epsilon.copy(), wl.epsilon.copy()
    ep[p] += 0.1
    em[p] -= 0.1
    fd.append((L(ep) - L(em)) / 0.2)
    ad.append(grad[p])
  fd, ad = np.array(fd), np.array(ad)
  err = np.linalg.norm(fd - ad) / np.linalg.norm(fd)
  print(f"c2 8 voxels: rel {err:.2e} at delta 0.1")
  print("fd(0.1)", fd)
  print("adjoint", ad)
  assert abs(fd1 - fd2) / abs(fd1) < 1e-3
  assert err_sign < 1e-3
  assert err_dir < 1e-2
  assert err < 1e-2


def test_c2_gradient_vs_tangent_linear_16_voxels(native):
  """c2's gate at 16 seeded voxels of the 50x50x6 design region.

  A central difference of the FP32 forward at delta-eps 1e-3 carries ~10%
  rounding noise on these derivatives (see the test above), so the
  reference here is the tangent-linear derivative of the same solve: one
  extra solve per voxel, driven at the voxel by the forward's own field
  increments (checked against FP64 central differences on the CPU in
  tests/test_tangent_cpu.py).  The adjoint gradient must match it to 1e-3
  relative (L2 over the 16 voxels)."""
  wl = workloads.design_c1(tt=20000)
  eps = torch.tensor(wl.epsilon, device=DEV, requires_grad=True)
  src = torch.as_tensor(wl.source, device=DEV)
  port = torch.as_tensor(workloads.port_profile(wl), device=DEV)
  F = pjz_gb300.field(eps, src, wl.omega, wl.source_pos, wl.sim_params)
  workloads.overlap_objective(F, wl, port).backward()
  grad = eps.grad.cpu().numpy()

  rng = np.random.default_rng(1)
  (bx, by, bz), (nx, ny, nz) = wl.design_box
  voxels = [(int(rng.integers(3)), bx + int(rng.integers(nx)),
             by + int(rng.integers(ny)), bz + int(rng.integers(nz)))
            for _ in range(16)]
  xo = workloads.output_plane(wl)
  _, _, yy, zz = wl.epsilon.shape
  dF = _tangent.field_voxel_jvp(wl.epsilon, src, wl.omega, wl.source_pos,
                                wl.sim_params, voxels, ((xo, 0, 0), (1, yy, zz)))
  p = port.to(torch.complex128)
  ov = (F.detach()[:, 1, xo].to(torch.complex128) * p).sum(dim=(-2, -1))
  dov = (dF[:, :, 1, 0].to(torch.complex128) * p).sum(dim=(-2, -1))
  tl = (2 * (torch.conj(ov)[None] * dov).real).sum(dim=-1).cpu().numpy()
  ad = np.array([grad[v] for v in voxels], np.float64)
  err = np.linalg.norm(ad - tl) / np.linalg.norm(tl)
  worst = np.max(np.abs(ad - tl) / np.abs(tl))
  print(f"c2 16 voxels, adjoint vs tangent-linear: rel-L2 {err:.2e}, worst "
        f"voxel {worst:.2e}")
  print("tangent", tl)
  print("adjoint", ad)
  assert err < 1e-3
