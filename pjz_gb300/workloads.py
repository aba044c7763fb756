"""Synthetic photonic workloads with the shapes of pjz's benchmark configs.

All lengths in cells at dx = 40 nm: lambda = 1.55 um is 38.75 cells, so
omega = 2 pi / 38.75; silicon eps 12.25, silica 2.085.  Geometry is seeded
(``numpy.random.default_rng``); no dataset is involved.

* ``waveguide_c0``: 128x128x32 domain, straight Si waveguide (10 cells wide,
  5.5 thick) along x, Gaussian current sheet (sigma 7.5 cells) at x=20,
  16-cell absorber, 8-cell z-PML, 2000 steps, one frequency.
* ``design_c1``: 512x512x64 domain, waveguide in/out along x through a
  central 50x50x6 design region of blurred uniform [2.085, 12.25] voxels,
  10000 steps, 5 frequencies over 1.50-1.60 um.

Each builder returns a :class:`Workload` holding pjz-level arguments
(``epsilon`` (3,xx,yy,zz) without the absorber padding, ``source``,
``omega``, ``source_pos``, ``SimParams``) whose domain equals the stated
grid (``LaunchParams.zz`` fixes the z extent).
"""

from typing import NamedTuple, Tuple

import numpy as np

from ._fdtdz import LaunchParams
from ._field import SimParams

EPS_SI = 12.25
EPS_SIO2 = 2.085
DX_NM = 40.0
# Strength of the 16-cell quadratic absorber (sigma_max = 1.28): weaker
# values let the guided mode reflect and keep the c1 run off steady state.
ABSORBER_COEFF = 5e-3


def omega_of(wavelength_um: float) -> float:
  return 2 * np.pi / (wavelength_um * 1000.0 / DX_NM)


class Workload(NamedTuple):
  name: str
  epsilon: np.ndarray        # (3, xx, yy, zz) float32, unpadded
  source: np.ndarray         # (2, 1, yy, zz) float32
  omega: np.ndarray          # (ww,)
  source_pos: int
  sim_params: SimParams
  domain: Tuple[int, int, int]
  design_box: Tuple[Tuple[int, int, int], Tuple[int, int, int]]  # origin, shape

  @property
  def cell_updates(self) -> int:
    X, Y, Z = self.domain
    return X * Y * Z * self.sim_params.tt


def _slab_fraction(n: int, lo: float, hi: float, offset: float) -> np.ndarray:
  """Fraction of each cell [k+offset-1/2, k+offset+1/2] inside [lo, hi]."""
  c = np.arange(n) + offset
  return np.clip(np.minimum(c + 0.5, hi) - np.maximum(c - 0.5, lo), 0, 1)


def _layered_eps(shape, core_y, core_z, core_x=None):
  """(3, X, Y, Z) silica with a silicon box; Yee offsets per component."""
  X, Y, Z = shape
  eps = np.empty((3, X, Y, Z), np.float64)
  for c in range(3):
    ox = 0.5 if c == 0 else 0.0
    oy = 0.5 if c == 1 else 0.0
    oz = 0.5 if c == 2 else 0.0
    fy = _slab_fraction(Y, *core_y, oy)
    fz = _slab_fraction(Z, *core_z, oz)
    fx = np.ones(X) if core_x is None else _slab_fraction(X, *core_x, ox)
    f = fx[:, None, None] * fy[None, :, None] * fz[None, None, :]
    eps[c] = EPS_SIO2 + (EPS_SI - EPS_SIO2) * f
  return eps


def _gaussian_sheet(Y, Z, yc, zc, sigma):
  y = np.arange(Y)[:, None] + 0.5 - yc  # Ey sits at y + 1/2
  z = np.arange(Z)[None, :] - zc
  return np.exp(-(y**2 + z**2) / (2 * sigma**2))


def _blur(a: np.ndarray, sigma: float) -> np.ndarray:
  """Separable Gaussian blur (reflect edges) over the first two axes."""
  r = int(np.ceil(3 * sigma))
  k = np.exp(-np.arange(-r, r + 1)**2 / (2 * sigma**2))
  k /= k.sum()
  out = a
  for ax in (0, 1):
    pad = [(0, 0)] * out.ndim
    pad[ax] = (r, r)
    p = np.pad(out, pad, mode="reflect")
    out = sum(k[i] * np.take(p, np.arange(i, i + out.shape[ax]), axis=ax)
              for i in range(2 * r + 1))
  return out


def waveguide_c0(tt: int = 2000, domain=(128, 128, 32), absorber: int = 16,
                 pml: int = 8) -> Workload:
  X, Y, Z = domain
  omega = np.array([omega_of(1.55)])
  zz_eps = Z - 2 * pml
  xx, yy = X - 2 * absorber, Y - 2 * absorber
  yc, zc = yy / 2, zz_eps / 2
  eps = _layered_eps((xx, yy, zz_eps), (yc - 5.0, yc + 5.0), (zc - 2.75, zc + 2.75))
  src = np.zeros((2, 1, yy, zz_eps), np.float32)
  src[0, 0] = _gaussian_sheet(yy, zz_eps, yc, zc, 7.5)
  ramp = float(omega[0] * 0.5 * 500)  # 500-step ramp in pjz's radian units
  sp = SimParams(omega_range=(float(omega[0]), float(omega[0])), tt=tt,
                 dt=0.5, source_ramp=ramp, source_delay=4.0,
                 absorption_padding=absorber, absorption_coeff=ABSORBER_COEFF,
                 pml_widths=(pml, pml), use_reduced_precision=False,
                 launch_params=LaunchParams(zz=Z))
  return Workload("c0 waveguide 128x128x32", eps.astype(np.float32), src,
                  omega, 20 - absorber, sp, tuple(domain),
                  ((0, 0, 0), (0, 0, 0)))


def design_problem(domain=(512, 512, 64), tt: int = 10000, wavelengths=None,
                   seed: int = 0, src_x: int = 20, design=(50, 50, 6),
                   absorber: int = 16, pml: int = 8, name: str = None) -> Workload:
  """Waveguide in and out along x through a central blurred random design
  region (voxels uniform in [2.085, 12.25], Gaussian blur sigma 2 cells,
  clipped), x-normal Gaussian sheet source at domain x = ``src_x``."""
  X, Y, Z = domain
  lam = np.atleast_1d(np.asarray(
      wavelengths if wavelengths is not None else [1.55], np.float64))
  omega = np.array([omega_of(l) for l in lam])
  zz_eps = Z - 2 * pml
  xx, yy = X - 2 * absorber, Y - 2 * absorber
  yc, zc = yy / 2, zz_eps / 2
  dx, dy, dz = design
  eps = _layered_eps((xx, yy, zz_eps), (yc - 5.0, yc + 5.0),
                     (zc - dz / 2, zc + dz / 2))
  rng = np.random.default_rng(seed)
  vox = rng.uniform(EPS_SIO2, EPS_SI, (dx, dy))
  vox = np.clip(_blur(vox, 2.0), EPS_SIO2, EPS_SI)
  x0, y0 = xx // 2 - dx // 2, yy // 2 - dy // 2
  z0 = int(round(zc - dz / 2))
  eps[:, x0:x0 + dx, y0:y0 + dy, z0:z0 + dz] = vox[None, :, :, None]
  src = np.zeros((2, 1, yy, zz_eps), np.float32)
  src[0, 0] = _gaussian_sheet(yy, zz_eps, yc, zc, 7.5)
  ramp = float(omega.mean() * 0.5 * 500)
  sp = SimParams(omega_range=(float(omega.min()), float(omega.max())), tt=tt,
                 dt=0.5, source_ramp=ramp, source_delay=4.0,
                 absorption_padding=absorber, absorption_coeff=ABSORBER_COEFF,
                 pml_widths=(pml, pml), use_reduced_precision=False,
                 launch_params=LaunchParams(zz=Z))
  return Workload(name or f"design {X}x{Y}x{Z}", eps.astype(np.float32), src,
                  omega, src_x - absorber, sp, tuple(domain),
                  ((x0, y0, z0), (dx, dy, dz)))


def design_c1(tt: int = 10000, domain=(512, 512, 64), absorber: int = 16,
              pml: int = 8, design=(50, 50, 6), ww: int = 5,
              seed: int = 0) -> Workload:
  X, Y, Z = domain
  lam = np.linspace(1.50, 1.60, ww) if ww > 1 else np.array([1.55])
  return design_problem(domain, tt, lam, seed, 20, design, absorber, pml,
                        name=f"c1 design {X}x{Y}x{Z}")


def batch_c3(n: int = 64, tt: int = 6000, seed: int = 2):
  """Config c3: ``n`` independent problems, x and y drawn from {256, 384,
  512}, z from {32, 48, 64}, each with its own blurred random design, its
  own source plane (domain x in [18, 40)) and 1-3 output frequencies evenly
  spread over 1.50-1.60 um; ``tt`` steps each."""
  rng = np.random.default_rng(seed)
  out = []
  for k in range(n):
    X, Y = (int(v) for v in rng.choice([256, 384, 512], 2))
    Z = int(rng.choice([32, 48, 64]))
    ww = int(rng.integers(1, 4))
    lam = np.linspace(1.50, 1.60, ww) if ww > 1 else np.array([1.55])
    out.append(design_problem((X, Y, Z), tt, lam, seed=1000 + k,
                              src_x=int(rng.integers(18, 40)),
                              name=f"c3[{k}] {X}x{Y}x{Z} ww={ww}"))
  return out


def port_profile(wl: Workload, sigma: float = 7.5) -> np.ndarray:
  """Gaussian port (sigma 7.5 cells = 300 nm) centred on the waveguide,
  ``(yy, zz)`` over the epsilon region's transverse plane."""
  _, _, yy, zz = wl.epsilon.shape
  return _gaussian_sheet(yy, zz, yy / 2, zz / 2, sigma).astype(np.float32)


def output_plane(wl: Workload) -> int:
  """x index (epsilon region frame) of the output monitor plane."""
  return wl.epsilon.shape[1] - 20


def overlap_objective(fields, wl: Workload, port=None, dtype=None):
  """c2 objective: ``sum_w |sum_{y,z} port * E_y(x_out)|^2`` of ``field``'s
  output ``(ww, 3, xx, yy, zz)`` (torch complex); ``dtype`` (e.g.
  complex128) sets the precision of the reduction."""
  import torch
  p = port if port is not None else torch.as_tensor(
      port_profile(wl), device=fields.device)
  e = fields[:, 1, output_plane(wl)]
  if dtype is not None:
    e, p = e.to(dtype), p.to(dtype)
  ov = (e * p).sum(dim=(-2, -1))
  return (ov.abs() ** 2).sum()
