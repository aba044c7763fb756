"""The synthetic workloads the bench and the tests use carry the stated
configurations: grid, steps, Courant number, wavelengths, waveguide and
design-region geometry and permittivities, absorber and PML widths, source
plane (c0 waveguide, c1 design, c3 batch, c4 8-port S-matrix)."""

import inspect

import numpy as np

from pjz_gb300 import smatrix, workloads
from pjz_gb300.workloads import EPS_SI, EPS_SIO2, omega_of


def test_constants():
  assert EPS_SI == 12.25 and EPS_SIO2 == 2.085
  # dx = 40 nm: 1.55 um is 38.75 cells.
  assert abs(omega_of(1.55) - 2 * np.pi / 38.75) < 1e-12


def test_c0_waveguide():
  wl = workloads.waveguide_c0()
  sp = wl.sim_params
  assert wl.domain == (128, 128, 32) and sp.tt == 2000 and sp.dt == 0.5
  assert np.allclose(wl.omega, [omega_of(1.55)])
  assert sp.absorption_padding == 16 and tuple(sp.pml_widths) == (8, 8)
  assert wl.source_pos + sp.absorption_padding == 20  # 20 cells from x = 0
  assert abs(sp.source_ramp - omega_of(1.55) * 0.5 * 500) < 1e-9
  eps = wl.epsilon
  assert eps.shape == (3, 96, 96, 16)
  assert eps.min() == np.float32(EPS_SIO2) and eps.max() == np.float32(EPS_SI)
  # Core 400 nm x 220 nm = 10 x 5.5 cells: the Ex profile through the core
  # sums to 10 full cells across y and 5.5 across z.
  frac = (eps[0] - EPS_SIO2) / (EPS_SI - EPS_SIO2)
  assert abs(frac[48].max(axis=1).sum() - 10.0) < 1e-5
  assert abs(frac[48].max(axis=0).sum() - 5.5) < 1e-5


def test_c1_design():
  wl = workloads.design_c1()
  sp = wl.sim_params
  assert wl.domain == (512, 512, 64) and sp.tt == 10000
  assert np.allclose(wl.omega, [omega_of(l) for l in np.linspace(1.50, 1.60, 5)])
  (x0, y0, z0), shape = wl.design_box
  assert shape == (50, 50, 6)
  d = wl.epsilon[:, x0:x0 + 50, y0:y0 + 50, z0:z0 + 6]
  assert d.min() >= np.float32(EPS_SIO2) and d.max() <= np.float32(EPS_SI)
  assert d.std() > 0.1  # blurred random voxels, not a constant
  assert np.array_equal(d[0], d[2]) and np.array_equal(d[..., 0], d[..., -1])


def test_c3_batch():
  probs = workloads.batch_c3(n=6, tt=6000)
  for wl in probs:
    X, Y, Z = wl.domain
    assert X in (256, 384, 512) and Y in (256, 384, 512) and Z in (32, 48, 64)
    assert wl.sim_params.tt == 6000 and 1 <= len(wl.omega) <= 3
    assert omega_of(1.60) - 1e-12 <= wl.omega.min() <= wl.omega.max() <= \
        omega_of(1.50) + 1e-12
  assert inspect.signature(workloads.batch_c3).parameters["n"].default == 64


def test_c4_smatrix_defaults_and_ports():
  par = inspect.signature(smatrix.build_c4).parameters
  assert par["domain"].default == (1024, 1024, 64)
  assert par["tt"].default == 12000
  assert tuple(par["wavelengths"].default) == (1.53, 1.55, 1.57)
  P = smatrix.build_c4(domain=(160, 160, 16), tt=100, device_cells=40, edge=12,
                       monitor_inset=6, window=8, pml=3)
  assert len(P.ports) == 8
  sides = [(p.axis, p.source < 80) for p in P.ports]
  assert all(sides.count(s) == 2 for s in set(sides)) and len(set(sides)) == 4
  assert np.allclose(P.omega, [omega_of(l) for l in (1.53, 1.55, 1.57)])
  assert P.target.shape == (8, 8) and not np.diag(P.target).any()
