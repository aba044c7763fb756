"""Pins the FP64 restatement of pjz's permittivity rendering
(``oracle/epsilon.py``) to pjz's own tests: every row of the four
``parametrize`` tables of ``tests/test_layers.py`` (extracted as text into
``tests/golden/reference_kats.json`` by ``tests/golden/make_kats.py``) is
rebuilt the way that test builds it and compared with its expected value,
within pytest.approx's default tolerance as there.  pjz calls the function
``render(layers, positions, grid_start, grid_end, m)`` in those tests."""

import itertools
import json
import os

import numpy as np
import pytest

from oracle import epsilon as eo

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")


def _table(kind):
  with open(GOLDEN) as f:
    (case,) = [c for c in json.load(f)["cases"] if c["kind"] == kind]
  rows = []
  for combo in itertools.product(*[t["rows"] for t in case["tables"]]):
    vals = {}
    for t, r in zip(case["tables"], combo):
      vals.update(zip(t["names"], r["values"]))
    rows.append(pytest.param(vals, id=combo[-1]["id"] or f"line{combo[-1]['line']}"))
  return rows


def _grid(zz):
  z = np.arange(zz, dtype=float)[:, None]
  return z + np.array([[-0.5, 0.0]]), z + np.array([[0.5, 1.0]])


@pytest.mark.parametrize("c", _table("render_simple"))
def test_simple(c):
  xx, yy, zz = c["domain"]
  m, (v0, v1), t = c["m"], c["vals"], c["thresh"]
  layer = v0 * np.ones((2, 2 * m * xx, 2 * m * yy))
  layer[1, t[0]:, t[1]:] = v1
  out = eo.render(layer, [t[2]], *_grid(zz), m)
  assert out[tuple(c["index"])] == pytest.approx(c["expected"])


@pytest.mark.parametrize("c", _table("render_x_threshold"))
def test_x_threshold(c):
  xx, yy, zz, m = 4, 3, 2, c["m"]
  layer = np.ones((1, 2 * m * xx, 2 * m * yy))
  layer[0, c["thresh"]:, :] = 3.0
  out = eo.render(layer, [], *_grid(zz), m)
  assert out[c["component"], c["index"], 0, 0] == pytest.approx(c["expected"])


@pytest.mark.parametrize("c", _table("render_z_threshold"))
def test_z_threshold(c):
  layer = np.ones((2, 2, 2))
  layer[1] = 3.0
  out = eo.render(layer, [c["thresh"]], *_grid(1), 1)
  assert out[c["component"], 0, 0, c["index"]] == pytest.approx(c["expected"])


@pytest.mark.parametrize("c", _table("render_corner"))
def test_corner(c):
  t = c["thresh"]
  layer = np.ones((2, 4, 4))
  layer[1, t[0]:, t[1]:] = 3.0
  out = eo.render(layer, [t[2]], *_grid(2), 1)
  assert out[tuple(c["index"])] == pytest.approx(c["expected"])


def test_tables_complete():
  counts = {k: len(_table(k)) for k in ("render_simple", "render_x_threshold",
                                        "render_z_threshold", "render_corner")}
  assert counts == {"render_simple": 18, "render_x_threshold": 32,
                    "render_z_threshold": 10, "render_corner": 33}


def test_uniform_and_simple_averaging():
  """A uniform stack renders its value everywhere; simple averaging is the
  occupancy-weighted mean of the layer means."""
  rng = np.random.default_rng(0)
  layers = np.full((3, 8, 12), 2.5)
  out = eo.epsilon(layers, [0.7, 2.2], 2, 4)
  assert out.shape == (3, 2, 3, 4)  # (2m xx, 2m yy) = (8, 12), m = 2
  np.testing.assert_allclose(out, 2.5, rtol=1e-14)
  layers = rng.uniform(1, 12, (2, 4, 4))
  s = eo.epsilon(layers, [0.25], 1, 1, use_simple_averaging=True)
  assert s.shape == (3, 2, 2, 1)
  # Ez at (x, y) = (1, 1) samples pixels 1..2 in x and y (its window is
  # shifted by half a cell); its cell [0, 1] in z holds layer 0 below the
  # interface at 0.25 and layer 1 above it.
  assert s[2, 1, 1, 0] == pytest.approx(0.25 * layers[0, 1:3, 1:3].mean()
                                        + 0.75 * layers[1, 1:3, 1:3].mean())
  # Ex at (0, 0) samples pixels 0..1 in x, and 0..1 in y with the edge
  # repeated (pixels 0, 0); its cell [-0.5, 0.5] holds 3/4 layer 0.
  win = lambda l: layers[l][0:2][:, [0, 0]].mean()
  assert s[0, 0, 0, 0] == pytest.approx(0.75 * win(0) + 0.25 * win(1))
