"""Pins the oracle: pjz's own golden vectors, and physics identities.

The reference's tests (``tests/test_boundaries.py``,
``tests/test_frequencies.py``, ``tests/test_waveforms.py`` of pjz) call names
that pjz no longer exports; their expected values are extracted as text into
``tests/golden/reference_kats.json`` (``tests/golden/make_kats.py``) and
checked here against both the oracle's restatement (``oracle/pjz_ref.py``) and
the product's mirror of the same helpers (``pjz_gb300/field.py``).
"""

import json
import os
import zlib

import numpy as np
import pytest

import oracle
from oracle import adjoint, pjz_ref, yee_numpy
from pjz_gb300 import _field as pf

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")


def _cases(kind):
  with open(GOLDEN) as f:
    return [c for c in json.load(f)["cases"] if c["kind"] == kind]


@pytest.mark.parametrize("impl", [pjz_ref.absorption_mask, pf._absorption_mask])
def test_absorption_mask_golden(impl):
  cases = _cases("absorption_mask")
  assert len(cases) == 6
  for c in cases:
    kw = c["kwargs"]
    mask = impl(kw["xx"], kw["yy"], kw["width"], kw["smoothness"])
    got = eval(c["index"], {"abs_mask": mask})
    np.testing.assert_array_equal(got, c["expected"],
                                  err_msg=f"{c['file']}:{c['line']}")


@pytest.mark.parametrize("impl", [pjz_ref.pml_sigma, pf._pml_sigma])
def test_pml_sigma_golden(impl):
  (c,) = _cases("pml_sigma")
  kw = c["kwargs"]
  got = impl(tuple(kw["pml_widths"]), kw["zz"], kw["ln_R"], kw["m"])
  np.testing.assert_array_almost_equal(got, c["expected"])


@pytest.mark.parametrize("impl", [pjz_ref.sampling_interval, pf._sampling_interval])
def test_sampling_interval_orthogonal(impl):
  # pjz tests/test_frequencies.py:8-18
  wmin, wmax, n, dt = 2 * np.pi / 40, 2 * np.pi / 36, 10, 0.5
  interval = impl(wmin, wmax, n, dt)
  ws = np.linspace(wmin, wmax, n)
  theta = ws * dt * interval * np.arange(2 * n)[:, None]
  a = np.hstack([np.sin(theta), np.cos(theta)])
  a /= np.linalg.norm(a, ord=2, axis=0)
  assert np.all(a.T @ a - np.eye(2 * n) < 1e-1)


def test_frequency_components_sign():
  # pjz tests/test_frequencies.py:21-30: sin -> -1j, cos -> 1.
  omegas = np.array([2 * np.pi / 40, 2 * np.pi / 39])
  steps = np.array([10, 20, 30, 40])
  dt = 0.5
  signal = np.sin(omegas[0] * dt * steps) + np.cos(omegas[1] * dt * steps)
  out = pjz_ref.frequency_components(signal[:, None, None, None, None], steps,
                                     omegas, dt)
  assert out[0].item() == pytest.approx(-1j, rel=1e-3)
  assert out[1].item() == pytest.approx(1, rel=1e-3)


@pytest.mark.parametrize("impl", [pjz_ref.ramped_sin, pf._ramped_sin])
def test_ramped_sin_golden(impl):
  # pjz tests/test_waveforms.py:8-14 (the current helper returns the complex
  # exponential; its imaginary part is the old real-valued ramped sine).
  (c,) = _cases("ramped_sin")
  omega, dt, tt = 2 * np.pi / 40, 0.5, 100000
  w = impl(np.array([omega]), c["kwargs"]["width"], c["kwargs"]["delay"], dt, tt)
  np.testing.assert_array_almost_equal(
      np.imag(w)[-10:], np.sin(omega * dt * np.arange(tt))[-10:])


def test_output_phases_pinv_projects_exactly():
  # pjz _field.py:214-216, 271-279: 2ww+1 samples resolve ww phasors.
  omega = np.array([0.15, 0.16, 0.17])
  dt, tt = 0.5, 4000
  interval = pjz_ref.sampling_interval(omega.min(), omega.max(), 3, dt)
  steps = pjz_ref.output_steps(tt, interval, 3)
  assert len(range(*steps)) == 7
  f = np.array([1 + 2j, -0.5j, 3.0])
  t = np.arange(*steps)
  sig = np.real(f[:, None] * np.exp(1j * omega[:, None] * dt * t)).sum(0)
  got = pjz_ref.frequency_components(sig, t, omega, dt)
  np.testing.assert_allclose(got, f, atol=1e-9)


def _small_problem(rng, X=12, Y=10, Z=16, tt=60, pml=(3, 4), alpha=0.05):
  eps = rng.uniform(1, 4, (3, X - 4, Y - 4, Z - 6)).astype(np.float32)
  mask = pjz_ref.absorption_mask(X, Y, 2, 0.05).astype(np.float32)
  sig = pjz_ref.pml_sigma(pml, Z, 0.5, 1.3).astype(np.float32)
  sf = rng.normal(size=(2, 1, Y, Z)).astype(np.float32)
  org, shp, prof = oracle.plane_source_box(sf, 5, (X, Y, Z))
  return dict(eps=eps, offset=(2, 2, 3), mask=mask, kappa=np.ones_like(sig),
              sigma=sig, alpha=alpha * np.ones_like(sig), dt=0.5, tt=tt,
              pml_widths=pml, source_origin=org, source_profile=prof,
              waveform=rng.normal(size=(tt, 2)).astype(np.float32),
              output_steps=(40, 60, 7))


def test_c_oracle_matches_numpy_fp64():
  kw = _small_problem(np.random.default_rng(0))
  c = oracle.run(**kw, precision="f64")
  snaps, fields = yee_numpy.run(**kw)
  np.testing.assert_allclose(c["out"], snaps, rtol=0, atol=1e-12 * np.abs(snaps).max())


def test_c_oracle_fp32_error_vs_fp64():
  kw = _small_problem(np.random.default_rng(1))
  a = oracle.run(**kw, precision="f32")["out"]
  b = oracle.run(**kw, precision="f64")["out"]
  assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-5


def test_projection_mode_equals_pinv_of_snapshots():
  kw = _small_problem(np.random.default_rng(2))
  snaps = oracle.run(**kw, precision="f64")["out"]
  w = np.random.default_rng(3).normal(size=(4, snaps.shape[0]))
  proj = oracle.run(**kw, precision="f64", mode="project", weights=w)["out"]
  np.testing.assert_allclose(proj, np.einsum("ij,j...->i...", w.astype(np.float32).astype(np.float64), snaps),
                             rtol=1e-12, atol=1e-12)


def test_energy_conserved_without_losses():
  """Lossless Yee (no absorber, no PML, zero walls) conserves
  sum(eps E^n.E^n) + sum(H^{n-1/2}.H^{n+1/2}) once the source is off."""
  rng = np.random.default_rng(4)
  X, Y, Z, tt = 10, 9, 8, 80
  eps = rng.uniform(1, 3, (3, X, Y, Z)).astype(np.float32)
  wave = np.zeros((tt, 1), np.float32)
  wave[:5, 0] = 1.0
  prof = rng.normal(size=(1, 3, 2, 2, 2)).astype(np.float32)
  zero = np.zeros((Z, 2), np.float32)
  base = dict(eps=eps, offset=(0, 0, 0), mask=np.zeros((3, X, Y), np.float32),
              kappa=np.ones((Z, 2), np.float32), sigma=zero, alpha=zero, dt=0.5,
              pml_widths=(0, 0), source_origin=(4, 4, 3), source_profile=prof,
              precision="f64", mode="none")
  energies = []
  f = np.zeros((6, X, Y, Z))
  for n in range(10, 60, 10):
    f1 = oracle.run(**base, tt=n, waveform=wave[:n], fields=np.zeros((6, X, Y, Z)))["fields"]
    f2 = oracle.run(**base, tt=n + 1, waveform=wave[:n + 1], fields=np.zeros((6, X, Y, Z)))["fields"]
    e = np.sum(eps * f1[:3] ** 2) + np.sum(f1[3:] * f2[3:])
    energies.append(e)
  energies = np.array(energies)
  assert energies[0] > 0
  np.testing.assert_allclose(energies, energies[0], rtol=1e-10)


def test_reciprocity_point_sources():
  """G_xz(a, b) == G_zx(b, a) for a symmetric (absorber-only) medium."""
  rng = np.random.default_rng(5)
  X, Y, Z, tt = 14, 12, 10, 120
  eps = rng.uniform(1, 3, (3, X, Y, Z)).astype(np.float32)
  mask = pjz_ref.absorption_mask(X, Y, 3, 0.05).astype(np.float32)
  zero = np.zeros((Z, 2), np.float32)
  wave = np.sin(0.3 * np.arange(tt)).astype(np.float32)[:, None]
  a, b = (4, 5, 3), (9, 6, 6)

  def run(at, comp):
    prof = np.zeros((1, 3, 1, 1, 1), np.float32)
    prof[0, comp] = 1.0
    r = oracle.run(eps=eps, offset=(0, 0, 0), mask=mask,
                   kappa=np.ones((Z, 2), np.float32), sigma=zero, alpha=zero,
                   dt=0.5, tt=tt, pml_widths=(0, 0), source_origin=at,
                   source_profile=prof, waveform=wave, precision="f64",
                   output_steps=(0, tt, 1), mode="snapshot")
    return r["out"]

  ea = run(a, 0)  # Jx at a
  eb = run(b, 2)  # Jz at b
  np.testing.assert_allclose(ea[:, 2, b[0], b[1], b[2]],
                             eb[:, 0, a[0], a[1], a[2]],
                             rtol=1e-9, atol=1e-12 * np.abs(ea).max())


def _cavity_modes(n):
  """Eigenpairs of the 1-D operator the Yee differences give on n cells:
  H from forward differences of E with E = 0 beyond the last cell, E from
  backward differences of H with H = 0 below the first (tridiag(-1, 2, -1)
  whose first diagonal entry is 1).  Mode m = 1..n: cos(k (i + 1/2)),
  k = pi (2m - 1) / (2n + 1), eigenvalue 4 sin^2(k / 2)."""
  i = np.arange(n) + 0.5
  for m in range(1, n + 1):
    k = np.pi * (2 * m - 1) / (2 * n + 1)
    yield np.cos(k * i), 4 * np.sin(k / 2) ** 2


def test_yee_dispersion_relation_of_cavity_modes():
  """With kappa = inf every z-layer is a 2-D Yee problem; the Ez part of
  each layer's cavity modes evolves, once the source is off, exactly as the
  leapfrog recurrence of the discrete dispersion relation
  a(n+1) + a(n-1) = 2 (1 - dt^2 lambda / (2 eps)) a(n), lambda the mode's
  eigenvalue of the discrete Laplacian."""
  X, Y, Z, tt, dt, eps_r = 9, 8, 2, 160, 0.5, 2.0
  wave = np.zeros((tt, 1), np.float32)
  wave[:3, 0] = (1.0, -1.0, 0.5)
  prof = np.zeros((1, 3, 1, 1, Z), np.float32)
  prof[0, 2] = 1.0  # Jz on one (x, y) column
  zero = np.zeros((Z, 2), np.float32)
  out = oracle.run(eps=np.full((3, X, Y, Z), eps_r, np.float32), offset=(0, 0, 0),
                   mask=np.zeros((3, X, Y), np.float32),
                   kappa=np.full((Z, 2), np.inf, np.float32), sigma=zero, alpha=zero,
                   dt=dt, tt=tt, pml_widths=(0, 0), source_origin=(3, 2, 0),
                   source_profile=prof, waveform=wave, precision="f64",
                   output_steps=(0, tt, 1), mode="snapshot")["out"]
  ez = out[:, 2, :, :, 0]
  mx, my = list(_cavity_modes(X)), list(_cavity_modes(Y))
  checked = 0
  for m, n in [(0, 0), (1, 2), (4, 1), (8, 7), (6, 3)]:
    (px, lx), (py, ly) = mx[m], my[n]
    a = np.einsum("txy,x,y->t", ez, px, py)
    c = 1 - dt * dt * (lx + ly) / (2 * eps_r)
    res = a[7:] + a[5:-2] - 2 * c * a[6:-1]
    assert np.abs(a).max() > 1e-3 * np.abs(ez).max()
    assert np.abs(res).max() < 1e-11 * np.abs(a).max(), (m, n)
    # The all-walls-zero sine modes are not this operator's modes.
    kx, ky = np.pi * (m + 1) / (X + 1), np.pi * (n + 1) / (Y + 1)
    b = np.einsum("txy,x,y->t", ez, np.sin(kx * np.arange(1, X + 1)),
                  np.sin(ky * np.arange(1, Y + 1)))
    cb = 1 - dt * dt * (4 * np.sin(kx / 2) ** 2 + 4 * np.sin(ky / 2) ** 2) / (2 * eps_r)
    assert np.abs(b[7:] + b[5:-2] - 2 * cb * b[6:-1]).max() > 1e-4 * np.abs(b).max()
    checked += 1
  assert checked == 5


def test_reciprocity_with_cpml_stretch():
  """The identity the adjoint rests on, A^T = S A S^-1 with S the CPML
  z-stretch of each E component: the response Ez(b) to Jx(a) equals
  S_x(a) / S_z(b) times the response Ex(a) to Jz(b) at every frequency
  (DTFT of fully decayed responses to a zero-mean pulse), while plain
  reciprocity fails once a and b sit at unlike depths of the z slabs."""
  X, Y, Z, tt, dt, pml = 14, 12, 16, 3000, 0.5, (4, 4)
  rng = np.random.default_rng(6)
  eps = rng.uniform(1, 3, (3, X, Y, Z)).astype(np.float32)
  mask = pjz_ref.absorption_mask(X, Y, 4, 0.05).astype(np.float32)
  sig = pjz_ref.pml_sigma(pml, Z, 0.5, 1.3).astype(np.float32)
  kappa = np.ones_like(sig)
  alpha = np.full_like(sig, 0.05)
  n = np.arange(tt)
  s = (n - 40) / 8.0
  wave = (-s * np.exp(-0.5 * s * s)).astype(np.float32)[:, None]
  a, b = (4, 5, 2), (9, 6, 14)  # both inside the z slabs, unlike depths

  def response(at, comp, probe, pcomp):
    prof = np.zeros((1, 3, 1, 1, 1), np.float32)
    prof[0, comp] = 1.0
    out = oracle.run(eps=eps, offset=(0, 0, 0), mask=mask, kappa=kappa, sigma=sig,
                     alpha=alpha, dt=dt, tt=tt, pml_widths=pml, source_origin=at,
                     source_profile=prof, waveform=wave, precision="f64",
                     output_steps=(0, tt, 1), mode="snapshot")["out"]
    return out[:, pcomp, probe[0], probe[1], probe[2]]

  zb_from_xa = response(a, 0, b, 2)
  xa_from_zb = response(b, 2, a, 0)
  peak = np.abs(zb_from_xa).max()
  assert np.abs(zb_from_xa[-100:]).max() < 1e-5 * peak  # decayed
  assert np.abs(zb_from_xa - xa_from_zb).max() > 0.1 * peak
  for w in (0.3, 0.5, 0.7):
    ph = np.exp(-1j * w * dt * n)
    S = adjoint.stretch(np.array([w]), dt, kappa, sig, alpha, pml)[0]
    ratio = S[0, a[2]] / S[2, b[2]]
    assert abs(ratio - 1) > 0.2
    got = (ph @ zb_from_xa) / (ph @ xa_from_zb)
    assert abs(got - ratio) < 2e-6 * abs(ratio), (w, got, ratio)


@pytest.mark.parametrize("orient", ["x", "y", "z"])
@pytest.mark.parametrize("pml,kinf", [((0, 0), False), ((3, 4), False),
                                       ((0, 5), False), ((2, 2), True)])
@pytest.mark.parametrize("full_region", [False, True])
def test_c_oracle_matches_numpy_fp64_variants(orient, pml, kinf, full_region):
  """The C oracle and the independent NumPy transcription agree (FP64) for
  every source orientation, z-PML layout (none, asymmetric, one-sided,
  kappa = inf) and epsilon region (offset inside the domain or the whole
  domain): snapshots and final fields."""
  rng = np.random.default_rng(zlib.crc32(repr((orient, pml, kinf, full_region)).encode()))
  X, Y, Z, tt = 12, 10, 16, 50
  if full_region:
    eps, offset = rng.uniform(1, 4, (3, X, Y, Z)), (0, 0, 0)
  else:
    eps, offset = rng.uniform(1, 4, (3, X - 4, Y - 4, Z - 6)), (2, 2, 3)
  sf = {"x": (rng.normal(size=(2, 1, Y, Z)), 5),
        "y": (rng.normal(size=(2, X, 1, Z)), 4),
        "z": (rng.normal(size=(2, 2, X, Y, 1)), 7)}[orient]
  org, shp, prof = oracle.plane_source_box(sf[0].astype(np.float32), sf[1], (X, Y, Z))
  sig = (pjz_ref.pml_sigma(pml, Z, 0.5, 1.3) if sum(pml) else
         np.zeros((Z, 2))).astype(np.float32)
  kappa = np.full_like(sig, np.inf) if kinf else np.ones_like(sig)
  kw = dict(eps=eps.astype(np.float32), offset=offset,
            mask=pjz_ref.absorption_mask(X, Y, 2, 0.05).astype(np.float32),
            kappa=kappa, sigma=sig, alpha=np.full_like(sig, 0.05), dt=0.5, tt=tt,
            pml_widths=pml, source_origin=org, source_profile=prof,
            waveform=rng.normal(size=(tt, 2)).astype(np.float32),
            output_steps=(30, 50, 5))
  c = oracle.run(**kw, precision="f64", fields=np.zeros((6, X, Y, Z)))
  snaps, fields = yee_numpy.run(**kw)
  scale = np.abs(fields).max()
  assert scale > 0 and np.abs(snaps).max() > 0
  np.testing.assert_allclose(c["out"], snaps, rtol=0, atol=1e-12 * scale)
  np.testing.assert_allclose(c["fields"], fields, rtol=0, atol=1e-12 * scale)


def test_oracle_binary16_rounding_matches_ieee():
  """The oracle's reduced-precision storage rounds to IEEE binary16 with
  round-to-nearest-even, subnormals and overflow to infinity, exactly as
  numpy's float16 conversion does (and as the GPU's cvt.rn.f16.f32)."""
  rng = np.random.default_rng(0)
  vals = (rng.normal(size=4000) * 10.0 ** rng.integers(-9, 6, 4000)).astype(np.float32)
  edge = np.float32([6.1e-5, 5.96e-8, 2.98e-8, 2.99e-8, 65504, 65519, 65520, 1e6,
                     -0.0, 0.0, np.inf, -np.inf, 1 + 2 ** -11, 1 + 3 * 2 ** -11])
  vals = np.concatenate([vals, edge])
  got = np.array([oracle.round_f16(v) for v in vals], np.float32)
  with np.errstate(over="ignore"):
    want = vals.astype(np.float16).astype(np.float32)
  assert np.array_equal(got, want)
  assert np.array_equal(np.signbit(got), np.signbit(want))
