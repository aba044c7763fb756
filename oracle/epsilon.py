"""FP64 NumPy restatement of pjz's permittivity rendering (test
infrastructure only).

Follows ``src/pjz/_epsilon.py`` of pjz: ``_render_single`` (:10-92),
``_render`` (:95-101) and ``epsilon`` (:104-155).  A layered stack of 2-D
profiles, magnified ``2m`` times in x and y, becomes the ``(3, xx, yy, zz)``
permittivity of the Yee cell: each component samples the cell it lives in
(Ex at x + 1/2, Ey at y + 1/2, Ez at z + 1/2), averages every layer over
that cell, and mixes the mean and the inverse mean of the inverse by the
diagonal of the interface projection (subpixel smoothing after Farjadpour
et al., Opt. Lett. 31, 2972 (2006)), with interface normals estimated from
least-squares slopes of the profiles inside the cell.  Only ``tests/``
import it.
"""

import numpy as np


def _shift_half_cell(layers, m, axis):
  """Profiles moved by half a cell (m pixels) towards +axis, the first m
  pixels repeating the edge: the window of a cell centred on an integer
  position along that axis."""
  n = layers.shape[axis]
  idx = np.concatenate([np.zeros(m, int), np.arange(n - m)])
  return np.take(layers, idx, axis=axis)


def _tile_stats(layers, m):
  """Per layer and 2m x 2m tile: mean, mean of the inverse, and the x and y
  slopes in cell units (12 mean(f u) for u the pixel-centre offset from the
  tile centre, the continuous least-squares normalisation)."""
  ll, px, py = layers.shape
  k = 2 * m
  t = layers.reshape(ll, px // k, k, py // k, k)
  u = (np.arange(k) - (m - 0.5)) / k
  mean = t.mean(axis=(2, 4))
  inv = (1.0 / t).mean(axis=(2, 4))
  gx = 12.0 * np.einsum("lxiyj,i->lxy", t, u) / (k * k)
  gy = 12.0 * np.einsum("lxiyj,j->lxy", t, u) / (k * k)
  return mean, inv, gx, gy


def _occupancy(layer_pos, lo, hi):
  """Fraction of each cell [lo, hi) every layer fills, (ll, zz), and the
  offset of the filled part's midpoint from the cell centre.  Layer l lies
  between interfaces l - 1 and l (the outer layers extend to infinity)."""
  edges = np.concatenate([[-np.inf], np.asarray(layer_pos, float), [np.inf]])
  bot = np.clip(edges[:-1, None], lo[None], hi[None])
  top = np.clip(edges[1:, None], lo[None], hi[None])
  frac = (top - bot) / (hi - lo)[None]
  mid = 0.5 * (bot + top) - 0.5 * (lo + hi)[None]
  return frac, mid


def render_component(layers, layer_pos, grid_start, grid_end, m, axis,
                     simple=False):
  """One Yee component (axis 0, 1, 2 for Ex, Ey, Ez): (xx, yy, zz)."""
  layers = np.asarray(layers, np.float64)
  for a in (0, 1):
    if axis != a:
      layers = _shift_half_cell(layers, m, 1 + a)
  col = 1 if axis == 2 else 0
  lo = np.asarray(grid_start, float)[:, col]
  hi = np.asarray(grid_end, float)[:, col]
  mean, inv, gx, gy = _tile_stats(layers, m)
  frac, mid = _occupancy(layer_pos, lo, hi)

  def over_layers(a, w):
    return np.einsum("lxy,lz->xyz", a, w)

  avg = over_layers(mean, frac)
  if simple:
    return avg
  inv_avg = over_layers(inv, frac)
  g = [over_layers(gx, frac), over_layers(gy, frac),
       over_layers(mean, frac * mid) / ((hi - lo) ** 2 / 12.0)]
  norm = g[0] ** 2 + g[1] ** 2 + g[2] ** 2
  p = g[axis] ** 2 / np.where(norm == 0, 1.0, norm)
  return 1.0 / (p * inv_avg + (1.0 - p) / avg)


def render(layers, layer_pos, grid_start, grid_end, m, simple=False):
  """(3, xx, yy, zz) permittivity for explicit z cell bounds: ``grid_start``
  / ``grid_end`` are (zz, 2), column 0 for Ex and Ey, column 1 for Ez."""
  return np.stack([render_component(layers, layer_pos, grid_start, grid_end, m,
                                    a, simple) for a in range(3)])


def epsilon(layers, interface_positions, magnification, zz,
            use_simple_averaging=False):
  """pjz's ``epsilon``: z cells [z - 1/2, z + 1/2] for Ex and Ey and
  [z, z + 1] for Ez."""
  z = np.arange(zz, dtype=float)[:, None]
  return render(layers, interface_positions, z + np.array([[-0.5, 0.0]]),
                z + np.array([[0.5, 1.0]]), magnification, use_simple_averaging)
