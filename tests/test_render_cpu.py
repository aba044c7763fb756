"""The permittivity rendering kernel's code on the CPU: ``tests/render_host.cpp``
runs the kernel's phases for every CTA with the same functions
(``pjz_gb300/csrc/render_kernel.cuh``), every read and write bounds-checked,
and is compared with the FP64 oracle (``oracle/epsilon.py``) on random
stacks of uneven shapes, and with the expected values of pjz's layer tests.
FP32 against FP64: relative tolerance 2e-5."""

import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import epsilon as eo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def host(tmp_path_factory):
  cxx = shutil.which("g++") or shutil.which("c++")
  if cxx is None:
    pytest.skip("no C++ compiler")
  lib = str(tmp_path_factory.mktemp("render") / "librender_host.so")
  subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared",
                  "-fPIC", "-Wall",
                  "-I", os.path.join(ROOT, "pjz_gb300", "csrc"),
                  os.path.join(ROOT, "tests", "render_host.cpp"), "-o", lib],
                 check=True)
  h = ctypes.CDLL(lib)
  P = ctypes.c_void_p
  I = ctypes.c_int
  h.render_host.argtypes = [P, I, I, I, I, I, P, I, I, I, P]
  h.render_host.restype = I
  h.render_owner_mismatches.argtypes = [P, I, I, I]
  h.render_owner_mismatches.restype = I
  return h


def render(host, layers, pos, m, zz, simple=False, finite=True, group=0, nxb=4):
  layers = np.ascontiguousarray(layers, np.float32)
  ll, px, py = layers.shape
  xx, yy = px // (2 * m), py // (2 * m)
  pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
  out = np.full((3, xx, yy, zz), np.nan, np.float32)
  bad = host.render_host(layers.ctypes.data, ll, xx, yy, zz, m,
                         pos.ctypes.data if pos.size else None, int(simple),
                         group, nxb, out.ctypes.data)
  assert bad == 0, "a read or write left its array"
  if finite:
    assert np.isfinite(out).all(), "an output was not written"
  return out


CASES = [  # (ll, xx, yy, zz, m, simple)
    (1, 3, 5, 4, 1, False), (2, 4, 33, 6, 2, False), (3, 7, 40, 9, 1, False),
    (4, 2, 65, 16, 3, False), (3, 5, 6, 7, 2, True), (16, 3, 3, 20, 1, False),
    (2, 1, 1, 1, 4, False), (5, 9, 31, 12, 2, True)]


@pytest.mark.parametrize("ll,xx,yy,zz,m,simple", CASES)
def test_matches_fp64_oracle(host, ll, xx, yy, zz, m, simple):
  rng = np.random.default_rng(ll * 1000 + xx * 100 + yy + zz)
  layers = rng.uniform(1.0, 12.25, (ll, 2 * m * xx, 2 * m * yy))
  # Interfaces inside, below and above the z range, some at cell edges.
  pos = np.sort(np.concatenate([rng.uniform(-1.0, zz + 1.0, max(ll - 3, 0)),
                                [0.0, 0.5 * zz][:min(2, ll - 1)]]))[:ll - 1]
  assert len(pos) == ll - 1
  got = render(host, layers, pos, m, zz, simple)
  want = eo.epsilon(layers.astype(np.float32).astype(np.float64),
                    pos.astype(np.float32).astype(np.float64), m, zz, simple)
  np.testing.assert_allclose(got, want, rtol=2e-5, atol=0)


def test_owner_by_comparison_matches_exact_fractions(host):
  """For sorted positions without NaN the kernel finds each z cell's
  filling layer by comparing positions with the cell bounds; it must name
  the same layer as the exact-fraction test (fraction == 1) for interfaces
  on cell edges and centres, ties (zero-thickness layers), infinities,
  huge values, and random positions."""
  rng = np.random.default_rng(5)
  cases = [[0.5, 1.0], [2.0, 2.0, 2.0], [-np.inf, 3.5, np.inf], [1e30, 2e30],
           [-1e30, 0.0], [4.5, 4.5, 5.0, 5.5], [0.25, 7.75]]
  for ll in range(2, 17):
    cases.append(np.sort(rng.uniform(-2, 12, ll - 1)))
    cases.append(np.sort(rng.integers(-2, 24, ll - 1) / 2.0))
    cases.append(np.sort(rng.integers(-8, 48, ll - 1) / 4.0))
  for pos in cases:
    pos = np.ascontiguousarray(pos, np.float32)
    assert host.render_owner_mismatches(pos.ctypes.data, len(pos) + 1, -3, 16) == 0, pos


@pytest.mark.parametrize("xx,nxb", [(7, 1), (7, 2), (7, 3), (9, 4), (1, 4)])
def test_x_cells_per_cta_give_the_same_floats(host, xx, nxb):
  """Several x cells per CTA (their patches share rows; the last CTA of a
  row may hold fewer) change no output bit."""
  rng = np.random.default_rng(xx * 10 + nxb)
  m, zz = 2, 10
  layers = rng.uniform(1.0, 12.25, (3, 2 * m * xx, 2 * m * 35))
  pos = np.array([2.5, 6.25], np.float32)
  want = render(host, layers, pos, m, zz, nxb=1)
  np.testing.assert_array_equal(render(host, layers, pos, m, zz, nxb=nxb), want)
  np.testing.assert_array_equal(render(host, layers, pos, m, zz, nxb=nxb, group=1),
                                want)


@pytest.mark.parametrize("ll,m", [(5, 2), (16, 1), (3, 3)])
def test_layer_groups_give_the_same_floats(host, ll, m):
  """Staging the layers in groups of any size (the library stages as many
  as fit its shared-memory budget) changes no output bit."""
  rng = np.random.default_rng(ll * 10 + m)
  xx, yy, zz = 3, 37, 11
  layers = rng.uniform(1.0, 12.25, (ll, 2 * m * xx, 2 * m * yy))
  pos = np.sort(rng.uniform(-1.0, zz + 1.0, ll - 1))
  want = render(host, layers, pos, m, zz)
  for g in range(1, ll):
    np.testing.assert_array_equal(render(host, layers, pos, m, zz, group=g), want)


def test_unsorted_positions_follow_the_oracle(host):
  """Positions out of order take the exact-fraction owner test; the result
  still follows the oracle (which applies pjz's formulas as they are)."""
  rng = np.random.default_rng(11)
  m, zz = 1, 10
  layers = rng.uniform(1.0, 12.0, (4, 2 * m * 3, 2 * m * 5))
  for pos in ([6.5, 2.25, 8.0], [3.0, np.nan, 5.5]):
    _unsorted_case(host, layers, np.array(pos, np.float32), m, zz)


def _unsorted_case(host, layers, pos, m, zz):
  got = render(host, layers, pos, m, zz, finite=False)
  with np.errstate(divide="ignore", invalid="ignore"):
    want = eo.epsilon(layers.astype(np.float32).astype(np.float64),
                      pos.astype(np.float64), m, zz, False)
  ok = np.isfinite(want)
  np.testing.assert_array_equal(np.isfinite(got), ok)
  np.testing.assert_allclose(got[ok], want[ok], rtol=2e-5, atol=1e-6)


def test_reference_layer_tables(host):
  """The four tables of pjz's tests/test_layers.py through the kernel code
  (the oracle's own test rebuilds them the same way)."""
  from test_epsilon_oracle import _table
  n = 0
  for c in (r.values[0] for r in _table("render_simple")):
    xx, yy, zz = c["domain"]
    m, (v0, v1), t = c["m"], c["vals"], c["thresh"]
    layer = v0 * np.ones((2, 2 * m * xx, 2 * m * yy))
    layer[1, t[0]:, t[1]:] = v1
    assert render(host, layer, [t[2]], m, zz)[tuple(c["index"])] == \
        pytest.approx(c["expected"], rel=1e-5)
    n += 1
  for c in (r.values[0] for r in _table("render_x_threshold")):
    m = c["m"]
    layer = np.ones((1, 2 * m * 4, 2 * m * 3))
    layer[0, c["thresh"]:, :] = 3.0
    assert render(host, layer, [], m, 2)[c["component"], c["index"], 0, 0] == \
        pytest.approx(c["expected"], rel=1e-5)
    n += 1
  for c in (r.values[0] for r in _table("render_z_threshold")):
    layer = np.ones((2, 2, 2))
    layer[1] = 3.0
    assert render(host, layer, [c["thresh"]], 1, 1)[c["component"], 0, 0,
                                                      c["index"]] == \
        pytest.approx(c["expected"], rel=1e-5)
    n += 1
  for c in (r.values[0] for r in _table("render_corner")):
    t = c["thresh"]
    layer = np.ones((2, 4, 4))
    layer[1, t[0]:, t[1]:] = 3.0
    assert render(host, layer, [t[2]], 1, 2)[tuple(c["index"])] == \
        pytest.approx(c["expected"], rel=1e-5)
    n += 1
  assert n == 93


@pytest.mark.parametrize("bad", [0.0, np.nan, np.inf])
@pytest.mark.parametrize("simple", [False, True])
def test_nonfinite_window_gives_the_oracle_nan_pattern(host, bad, simple):
  """A zero, NaN or infinite pixel in one layer: pjz's einsum multiplies
  that layer's statistics by the zero fractions of the cells other layers
  fill (0 * inf = NaN), so the whole column follows; the one-layer
  shortcut must not hide it."""
  rng = np.random.default_rng(3)
  m, zz = 1, 8
  layers = rng.uniform(2.0, 12.0, (3, 2 * m * 5, 2 * m * 6)).astype(np.float32)
  layers[0, 4, 5] = bad
  pos = np.array([2.5, 5.0], np.float32)
  with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
    want = eo.epsilon(layers.astype(np.float64), pos.astype(np.float64), m, zz,
                      simple)
  got = render(host, layers, pos, m, zz, simple, finite=False)
  # With simple averaging only the mean enters, which a zero pixel keeps
  # finite.
  assert np.isfinite(want).all() == (simple and bad == 0.0)
  np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
  np.testing.assert_array_equal(np.isinf(got), np.isinf(want))
  ok = np.isfinite(want)
  np.testing.assert_allclose(got[ok], want[ok], rtol=2e-5, atol=0)


@pytest.mark.parametrize("shape,pos,m,msg", [
    ((2, 6, 8), [0.5], 2, "whole cells"),
    ((2, 8, 8), [0.5, 1.0], 2, "interface positions"),
    ((8, 8), [], 2, "layers must be"),
])
def test_epsilon_argument_errors(shape, pos, m, msg):
  """pjz_gb300.epsilon refuses bad shapes before any device work."""
  import pjz_gb300
  with pytest.raises(ValueError, match=msg):
    pjz_gb300.epsilon(np.ones(shape, np.float32), pos, m, 4)
