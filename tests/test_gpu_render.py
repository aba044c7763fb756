"""pjz's permittivity rendering on the GPU (``pjz_gb300.epsilon``, the native
render kernel): against the FP64 oracle on uneven shapes (relative 2e-5,
FP32 against FP64), against every expected value of pjz's layer tests, and
against the host emulation of the same kernel code on a production-size
stack (512 x 512 cells at 2x magnification, 3 layers, zz 64; relative
1e-6), and the NaN pattern of a stack with a zero or NaN pixel."""

import numpy as np
import pytest
import torch

import pjz_gb300
from oracle import epsilon as eo
from test_epsilon_oracle import _table
from test_render_cpu import host, render  # noqa: F401 (fixture)

pytestmark = pytest.mark.gpu

CASES = [(1, 3, 5, 4, 1, False), (2, 4, 33, 6, 2, False), (3, 7, 40, 9, 1, False),
         (4, 2, 65, 16, 3, False), (3, 5, 6, 7, 2, True), (16, 3, 3, 20, 1, False)]


def _stack(ll, xx, yy, zz, m):
  rng = np.random.default_rng(ll * 1000 + xx * 100 + yy + zz)
  layers = rng.uniform(1.0, 12.25, (ll, 2 * m * xx, 2 * m * yy)).astype(np.float32)
  pos = np.sort(np.concatenate([rng.uniform(-1.0, zz + 1.0, max(ll - 3, 0)),
                                [0.0, 0.5 * zz][:min(2, ll - 1)]]))[:ll - 1]
  return layers, pos.astype(np.float32)


def _gpu(layers, pos, m, zz, simple=False):
  out = pjz_gb300.epsilon(torch.as_tensor(layers, device="cuda"), pos, m, zz, simple)
  torch.cuda.synchronize()
  return out.cpu().numpy()


@pytest.mark.parametrize("ll,xx,yy,zz,m,simple", CASES)
def test_gpu_matches_fp64_oracle(native, ll, xx, yy, zz, m, simple):
  layers, pos = _stack(ll, xx, yy, zz, m)
  want = eo.epsilon(layers.astype(np.float64), pos.astype(np.float64), m, zz, simple)
  np.testing.assert_allclose(_gpu(layers, pos, m, zz, simple), want, rtol=2e-5,
                             atol=0)


def test_gpu_reference_layer_tables(native):
  n = 0
  for c in (r.values[0] for r in _table("render_corner")):
    t = c["thresh"]
    layer = np.ones((2, 4, 4), np.float32)
    layer[1, t[0]:, t[1]:] = 3.0
    assert _gpu(layer, [t[2]], 1, 2)[tuple(c["index"])] == \
        pytest.approx(c["expected"], rel=1e-5)
    n += 1
  for c in (r.values[0] for r in _table("render_x_threshold")):
    m = c["m"]
    layer = np.ones((1, 2 * m * 4, 2 * m * 3), np.float32)
    layer[0, c["thresh"]:, :] = 3.0
    assert _gpu(layer, [], m, 2)[c["component"], c["index"], 0, 0] == \
        pytest.approx(c["expected"], rel=1e-5)
    n += 1
  for c in (r.values[0] for r in _table("render_z_threshold")):
    layer = np.ones((2, 2, 2), np.float32)
    layer[1] = 3.0
    assert _gpu(layer, [c["thresh"]], 1, 1)[c["component"], 0, 0, c["index"]] == \
        pytest.approx(c["expected"], rel=1e-5)
    n += 1
  for c in (r.values[0] for r in _table("render_simple")):
    xx, yy, zz = c["domain"]
    m, (v0, v1), t = c["m"], c["vals"], c["thresh"]
    layer = v0 * np.ones((2, 2 * m * xx, 2 * m * yy), np.float32)
    layer[1, t[0]:, t[1]:] = v1
    assert _gpu(layer, [t[2]], m, zz)[tuple(c["index"])] == \
        pytest.approx(c["expected"], rel=1e-5)
    n += 1
  assert n == 93


def test_gpu_matches_host_emulation_production_size(native, host):
  rng = np.random.default_rng(7)
  m, zz = 2, 64
  layers = rng.uniform(2.085, 12.25, (3, 2 * m * 512, 2 * m * 512)).astype(np.float32)
  pos = np.array([28.5, 35.25], np.float32)
  d = torch.as_tensor(layers, device="cuda")
  out = torch.empty((3, 512, 512, zz), device="cuda")
  pjz_gb300.epsilon(d, pos, m, zz, out=out)  # warm-up
  e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
  e0.record()
  pjz_gb300.epsilon(d, pos, m, zz, out=out)
  e1.record()
  torch.cuda.synchronize()
  print(f"render 512x512x64 (3 layers, 2x): {e0.elapsed_time(e1):.3f} ms")
  np.testing.assert_allclose(out.cpu().numpy(), render(host, layers, pos, m, zz),
                             rtol=1e-6, atol=0)


@pytest.mark.parametrize("bad", [0.0, np.nan])
@pytest.mark.parametrize("simple", [False, True])
def test_gpu_nonfinite_window_matches_oracle_pattern(native, bad, simple):
  """A zero pixel (infinite inverse) or a NaN pixel in one layer gives the
  NaN / inf pattern of pjz's einsum (0 * inf = NaN) in every z cell of that
  column, including cells another layer fills."""
  rng = np.random.default_rng(3)
  m, zz = 1, 8
  layers = rng.uniform(2.0, 12.0, (3, 2 * m * 5, 2 * m * 6)).astype(np.float32)
  layers[0, 4, 5] = bad
  pos = np.array([2.5, 5.0], np.float32)
  with np.errstate(divide="ignore", invalid="ignore"):
    want = eo.epsilon(layers.astype(np.float64), pos.astype(np.float64), m, zz,
                      simple)
  got = _gpu(layers, pos, m, zz, simple)
  np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
  np.testing.assert_array_equal(np.isinf(got), np.isinf(want))
  ok = np.isfinite(want)
  np.testing.assert_allclose(got[ok], want[ok], rtol=2e-5, atol=0)


@pytest.mark.parametrize("pos", [[6.5, 2.25, 8.0], [3.0, float("nan"), 5.5]])
def test_gpu_unordered_or_nan_positions_take_the_full_mix(native, host, pos):
  """Out-of-order or NaN interface positions: no cell has a single owner,
  every cell takes the full mix -- bit-equal to the host emulation and
  following the oracle (NaN where it is NaN)."""
  rng = np.random.default_rng(12)
  m, zz = 2, 12
  layers = rng.uniform(1.0, 12.0, (4, 2 * m * 5, 2 * m * 37)).astype(np.float32)
  pos = np.array(pos, np.float32)
  got = _gpu(layers, pos, m, zz)
  np.testing.assert_array_equal(got, render(host, layers, pos, m, zz, finite=False))
  with np.errstate(divide="ignore", invalid="ignore"):
    want = eo.epsilon(layers.astype(np.float64), pos.astype(np.float64), m, zz, False)
  ok = np.isfinite(want)
  np.testing.assert_array_equal(np.isfinite(got), ok)
  np.testing.assert_allclose(got[ok], want[ok], rtol=2e-5, atol=1e-6)
