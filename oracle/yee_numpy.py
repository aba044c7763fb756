"""Vectorised NumPy FP64 Yee transcription (test infrastructure only).

An independent second restatement of the update in ``yee.c`` (same
conventions, see that file's header), written with whole-array slicing rather
than per-cell loops.  It exists to cross-check the C oracle on small grids;
it is far too slow for production sizes.  Only ``tests/`` import it.
"""

import numpy as np


def _pml_coeffs(kappa, sigma, alpha, dt):
  """CPML (ik, b, c) per z for one column (Roden-Gedney recursion)."""
  kappa = np.asarray(kappa, np.float64)
  sigma = np.asarray(sigma, np.float64)
  alpha = np.asarray(alpha, np.float64)
  inf = np.isinf(kappa)
  ik = np.where(inf, 0.0, 1.0 / np.where(inf, 1.0, kappa))
  kk = np.where(inf, 1.0, kappa)
  b = np.exp(-(np.where(inf, 0.0, sigma / kk) + alpha) * dt)
  den = sigma * kk + kk * kk * alpha
  c = np.where((sigma == 0) | inf, 0.0,
               sigma * (b - 1.0) / np.where(den == 0, 1.0, den))
  return ik, b, c


def run(*, eps, offset, mask, kappa, sigma, alpha, dt, tt, pml_widths,
        source_origin, source_profile, waveform, output_steps):
  """Returns (E snapshots (ns,3,region), final fields (6,X,Y,Z)) in FP64."""
  _, X, Y = mask.shape
  Z = kappa.shape[0]
  ox, oy, oz = offset
  rx, ry, rz = eps.shape[1:]
  xi = np.clip(np.arange(X) - ox, 0, rx - 1)
  yi = np.clip(np.arange(Y) - oy, 0, ry - 1)
  zi = np.clip(np.arange(Z) - oz, 0, rz - 1)
  e = np.asarray(eps, np.float64)[:, xi][:, :, yi][:, :, :, zi]
  s = np.asarray(mask, np.float64)[..., None]
  cb = dt / (e + s * (0.5 * dt))
  ike, be, ce = _pml_coeffs(kappa[:, 0], sigma[:, 0], alpha[:, 0], dt)
  ikh, bh, ch = _pml_coeffs(kappa[:, 1], sigma[:, 1], alpha[:, 1], dt)
  lo, hi = pml_widths
  inpml = np.zeros(Z, bool)
  inpml[:lo] = True
  if hi:
    inpml[Z - hi:] = True
  ce = np.where(inpml, ce, 0.0)
  ch = np.where(inpml, ch, 0.0)

  E = np.zeros((3, X, Y, Z))
  H = np.zeros((3, X, Y, Z))
  psi_h = np.zeros((2, X, Y, Z))
  psi_e = np.zeros((2, X, Y, Z))

  def fwd(a, axis):  # a[i+1] - a[i], zero beyond the far edge
    out = -a.copy()
    sl_dst = [slice(None)] * 3
    sl_src = [slice(None)] * 3
    sl_dst[axis] = slice(0, -1)
    sl_src[axis] = slice(1, None)
    out[tuple(sl_dst)] += a[tuple(sl_src)]
    return out

  def bwd(a, axis):  # a[i] - a[i-1], zero before the near edge
    out = a.copy()
    sl_dst = [slice(None)] * 3
    sl_src = [slice(None)] * 3
    sl_dst[axis] = slice(1, None)
    sl_src[axis] = slice(0, -1)
    out[tuple(sl_dst)] -= a[tuple(sl_src)]
    return out

  prof = np.asarray(source_profile, np.float64)
  sx, sy, sz = source_origin
  nx, ny, nz = prof.shape[2:]
  steps = range(*output_steps)
  snaps = []
  for n in range(tt):
    dEy_z, dEx_z = fwd(E[1], 2), fwd(E[0], 2)
    psi_h[0] = bh * psi_h[0] + ch * dEy_z
    psi_h[1] = bh * psi_h[1] + ch * dEx_z
    zEy = dEy_z * ikh + psi_h[0]
    zEx = dEx_z * ikh + psi_h[1]
    H[0] -= dt * (fwd(E[2], 1) - zEy)
    H[1] -= dt * (zEx - fwd(E[2], 0))
    H[2] -= dt * (fwd(E[1], 0) - fwd(E[0], 1))

    dHy_z, dHx_z = bwd(H[1], 2), bwd(H[0], 2)
    psi_e[0] = be * psi_e[0] + ce * dHy_z
    psi_e[1] = be * psi_e[1] + ce * dHx_z
    zHy = dHy_z * ike + psi_e[0]
    zHx = dHx_z * ike + psi_e[1]
    curl = np.stack([bwd(H[2], 1) - zHy, zHx - bwd(H[2], 0),
                     bwd(H[1], 0) - bwd(H[0], 1)])
    J = np.tensordot(np.asarray(waveform[n], np.float64), prof, axes=(0, 0))
    curl[:, sx:sx + nx, sy:sy + ny, sz:sz + nz] -= J
    E += cb * (curl - s * E)
    if n in steps:
      snaps.append(E[:, ox:ox + rx, oy:oy + ry, oz:oz + rz].copy())
  snaps = np.stack(snaps) if snaps else np.zeros((0, 3, rx, ry, rz))
  return snaps, np.concatenate([E, H])
