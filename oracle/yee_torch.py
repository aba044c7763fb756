"""FP32 torch-eager Yee restatement on the CPU (CPU baseline only).

The update of ``yee.c`` (same conventions, see that file's header) written
with whole-array torch operations on CPU tensors, the way a user would port
the update to eager PyTorch: forward/backward differences into preallocated
buffers, in-place updates, z-CPML state kept only in the PML slabs.  It is
timed beside the C oracle as a second CPU baseline; ``tests/`` check it
against the C oracle.  FP32 throughout, so it agrees with the oracle to
rounding, not bit for bit (the operation order differs).
"""

import numpy as np
import torch

from .yee_numpy import _pml_coeffs


def _fwd(out, a, axis):
  """out = a[i+1] - a[i] along `axis`, zero beyond the far edge."""
  n = a.shape[axis]
  torch.neg(a, out=out)
  out.narrow(axis, 0, n - 1).add_(a.narrow(axis, 1, n - 1))
  return out


def _bwd(out, a, axis):
  """out = a[i] - a[i-1] along `axis`, zero before the near edge."""
  n = a.shape[axis]
  out.copy_(a)
  out.narrow(axis, 1, n - 1).sub_(a.narrow(axis, 0, n - 1))
  return out


def _f32(v):
  return torch.from_numpy(np.ascontiguousarray(v, np.float32))


def run(*, eps, offset, mask, kappa, sigma, alpha, dt, tt, pml_widths,
        source_origin, source_profile, waveform, threads=0):
  """Runs `tt` steps from the zero state; returns the final fields
  (6, X, Y, Z) as float32 NumPy (E then H)."""
  if threads:
    torch.set_num_threads(threads)
  _, X, Y = mask.shape
  Z = kappa.shape[0]
  ox, oy, oz = offset
  rx, ry, rz = eps.shape[1:]
  xi = np.clip(np.arange(X) - ox, 0, rx - 1)
  yi = np.clip(np.arange(Y) - oy, 0, ry - 1)
  zi = np.clip(np.arange(Z) - oz, 0, rz - 1)
  e = _f32(np.asarray(eps, np.float32)[:, xi][:, :, yi][:, :, :, zi])
  s = _f32(mask)[..., None]                         # (3, X, Y, 1)
  cb = dt / (e + s * (0.5 * dt))
  ike, be, ce = (_f32(v) for v in _pml_coeffs(kappa[:, 0], sigma[:, 0],
                                              alpha[:, 0], dt))
  ikh, bh, ch = (_f32(v) for v in _pml_coeffs(kappa[:, 1], sigma[:, 1],
                                              alpha[:, 1], dt))
  lo, hi = pml_widths
  slabs = [(0, lo)] if lo else []
  if hi:
    slabs.append((Z - hi, hi))
  psi_h = [torch.zeros(2, X, Y, w) for _, w in slabs]
  psi_e = [torch.zeros(2, X, Y, w) for _, w in slabs]

  E = torch.zeros(3, X, Y, Z)
  H = torch.zeros(3, X, Y, Z)
  t1, t2, t3, t4 = (torch.empty(X, Y, Z) for _ in range(4))
  prof = _f32(source_profile)
  sx, sy, sz = source_origin
  nx, ny, nz = prof.shape[2:]
  wave = _f32(waveform)

  for n in range(tt):
    # H^{n+1/2}: forward differences of E.
    _fwd(t1, E[1], 2)                       # dEy/dz
    _fwd(t2, E[0], 2)                       # dEx/dz
    for (z0, w), p in zip(slabs, psi_h):
      zs = slice(z0, z0 + w)
      p[0].mul_(bh[zs]).addcmul_(ch[zs], t1[..., zs])
      p[1].mul_(bh[zs]).addcmul_(ch[zs], t2[..., zs])
    t1.mul_(ikh)
    t2.mul_(ikh)
    for (z0, w), p in zip(slabs, psi_h):
      t1[..., z0:z0 + w].add_(p[0])
      t2[..., z0:z0 + w].add_(p[1])
    H[0].sub_(_fwd(t3, E[2], 1).sub_(t1), alpha=dt)
    H[1].sub_(t2.sub_(_fwd(t3, E[2], 0)), alpha=dt)
    H[2].sub_(_fwd(t3, E[1], 0).sub_(_fwd(t4, E[0], 1)), alpha=dt)

    # E^{n+1}: backward differences of H, source, absorber.
    _bwd(t1, H[1], 2)                       # dHy/dz
    _bwd(t2, H[0], 2)                       # dHx/dz
    for (z0, w), p in zip(slabs, psi_e):
      zs = slice(z0, z0 + w)
      p[0].mul_(be[zs]).addcmul_(ce[zs], t1[..., zs])
      p[1].mul_(be[zs]).addcmul_(ce[zs], t2[..., zs])
    t1.mul_(ike)
    t2.mul_(ike)
    for (z0, w), p in zip(slabs, psi_e):
      t1[..., z0:z0 + w].add_(p[0])
      t2[..., z0:z0 + w].add_(p[1])
    c0 = _bwd(t3, H[2], 1).sub_(t1)         # dHz/dy - zHy
    c1 = t2.sub_(_bwd(t1, H[2], 0))         # zHx - dHz/dx
    c2 = _bwd(t1, H[1], 0).sub_(_bwd(t4, H[0], 1))
    J = torch.tensordot(wave[n], prof, dims=([0], [0]))
    for c, cur in enumerate((c0, c1, c2)):
      cur[sx:sx + nx, sy:sy + ny, sz:sz + nz].sub_(J[c])
      cur.addcmul_(s[c], E[c], value=-1.0)
      E[c].addcmul_(cb[c], cur)
  return torch.cat([E, H]).numpy()
