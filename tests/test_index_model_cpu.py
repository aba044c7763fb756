"""Bounds and alignment model of the streamed kernels' bulk copies (CPU).

compute-sanitizer is closed on this machine, and a bulk copy whose address or
size is not a multiple of 16 bytes, or that leaves its buffer, faults the
GPU.  This test restates the shared-memory layout and the copies of
`csrc/stream_kernel.cuh` (one step per launch, with and without
ring-carried source rows) and `csrc/stream2_kernel.cuh` (two steps per
launch) -- every ring-slot fill and every result store, for every tile,
segment and plane -- and checks on a grid of shapes that each one is 16-byte
aligned on both ends, a whole number of 16-byte units, inside its region of
the slot, and inside its global array.  It mirrors the kernels' index
arithmetic line for line; a kernel change to that arithmetic must change
this model with it.
"""

import itertools

import pytest

SMEM_BUDGET = 220 * 1024       # tile selection budget of the host
SMEM_MAX = 227 * 1024 - 2048   # ring-carried source rows


def r4(v):
  return (v + 3) & ~3


class Copies:
  """Collects violations of one copy list."""

  def __init__(self):
    self.bad = []
    self.count = 0

  def smem(self, what, off, nfl, lo, hi):
    """Shared-memory span [off, off + nfl) floats inside region [lo, hi)."""
    self.count += 1
    if off % 4 or nfl % 4 or nfl <= 0 or off < lo or off + nfl > hi:
      self.bad.append((what, "smem", off, nfl, lo, hi))

  def gmem(self, what, off, nfl, size):
    """Global span [off, off + nfl) floats inside an array of `size` floats
    whose base is 16-byte aligned."""
    if off % 4 or nfl % 4 or off < 0 or off + nfl > size:
      self.bad.append((what, "gmem", off, nfl, size))


def one_step(X, Y, Z, P, TY, S, seg_x, src=None):
  """Copies of yee_stream_kernel for one launch; `src` = (sx0, sy0, sz0, snx,
  sny, snz, ncols) of the source box or None."""
  Pp = r4(P)
  Yp = r4(Y)
  N, YZ, PXY = X * Y * Z, Y * Z, X * Y * Pp
  RE, RH, MT = TY + 2, TY + 1, r4(TY) + 8
  e_off = 0
  h_off = e_off + 3 * RE * Z
  c_off = h_off + 3 * RH * Z
  m_off = c_off + 3 * TY * Z
  p_off = m_off + 3 * MT
  s_off = p_off + 4 * RH * Pp

  def smem_bytes(sw):
    stage = s_off + sw
    floats = S * stage + 2 * 3 * RH * Z + 2 * 3 * TY * Z + 2 * 4 * TY * Pp
    return floats * 4 + (2 * S + 2) * 8 + 16

  if smem_bytes(0) > SMEM_BUDGET:  # the host refuses the tile
    return None
  sw = 0
  if src is not None:  # the host carries the source rows only if they fit
    sx0, sy0, sz0, snx, sny, snz, snc = src
    srowf = snc * 3 * snz
    rows = min(TY, sny)
    if srowf % 4 == 0 and smem_bytes(rows * srowf) <= SMEM_MAX:
      sw = rows * srowf
  stage = s_off + sw
  hn = S * stage
  en = hn + 2 * 3 * RH * Z
  pn = en + 2 * 3 * TY * Z
  end = pn + 2 * 4 * TY * Pp
  cp = Copies()
  for tile in range((Y + TY - 1) // TY):
    y0 = tile * TY
    ey_lo, ey_hi = max(y0 - 1, 0), min(y0 + TY + 1, Y)
    hy_hi = min(y0 + TY, Y)
    nrows = hy_hi - y0
    erow0 = ey_lo - (y0 - 1)
    ma, mb = y0 & ~3, min(r4(y0 + TY), Yp)
    for seg in range((X + seg_x - 1) // seg_x):
      xs = seg * seg_x
      xe = min(X, xs + seg_x)
      x0 = xs - 1 if xs > 0 else 0
      xlast = min(xe, X - 1)
      for xp in range(x0, xlast + 1):
        fullp = xp < xe
        for slot in range(min(S, 2)):  # slot placement repeats with period S
          st = slot * stage
          for c in range(3):
            cp.smem("E", st + e_off + c * RE * Z + erow0 * Z, (ey_hi - ey_lo) * Z,
                    st + e_off + c * RE * Z, st + e_off + (c + 1) * RE * Z)
          if not fullp:
            continue
          for c in range(3):
            cp.smem("H", st + h_off + c * RH * Z + erow0 * Z, (hy_hi - ey_lo) * Z,
                    st + h_off + c * RH * Z, st + h_off + (c + 1) * RH * Z)
            cp.smem("cb", st + c_off + c * TY * Z, nrows * Z,
                    st + c_off + c * TY * Z, st + c_off + (c + 1) * TY * Z)
            cp.smem("mask", st + m_off + c * MT, mb - ma, st + m_off + c * MT,
                    st + m_off + (c + 1) * MT)
          if Pp:
            for c in range(4):
              cp.smem("psi", st + p_off + c * RH * Pp + erow0 * Pp,
                      (hy_hi - ey_lo) * Pp, st + p_off + c * RH * Pp,
                      st + p_off + (c + 1) * RH * Pp)
        for c in range(3):
          cp.gmem("E", c * N + xp * YZ + ey_lo * Z, (ey_hi - ey_lo) * Z, 6 * N)
          if fullp:
            cp.gmem("H", (3 + c) * N + xp * YZ + ey_lo * Z, (hy_hi - ey_lo) * Z, 6 * N)
            cp.gmem("cb", c * N + xp * YZ + y0 * Z, nrows * Z, 3 * N)
            cp.gmem("mask", (xp * 3 + c) * Yp + ma, mb - ma, X * 3 * Yp)
        if fullp and Pp:
          for c in range(4):
            cp.gmem("psi", c * PXY + (xp * Y + ey_lo) * Pp, (hy_hi - ey_lo) * Pp,
                    4 * PXY)
        if fullp and sw:
          srow0 = max(y0, sy0)
          nsrow = min(min(y0 + TY, Y), sy0 + sny) - srow0
          if nsrow > 0 and sx0 <= xp < sx0 + snx:
            cp.smem("src", s_off, nsrow * srowf, s_off, s_off + sw)
            cp.gmem("src", ((xp - sx0) * sny + (srow0 - sy0)) * srowf,
                    nsrow * srowf, snc * 3 * snx * sny * snz)
      for x in range(xs, xe):  # result stores
        for b in range(2):
          for c in range(3):
            cp.smem("H out", hn + b * 3 * RH * Z + c * RH * Z + Z, nrows * Z,
                    hn, en)
            cp.smem("E out", en + b * 3 * TY * Z + c * TY * Z, nrows * Z, en, pn)
          if Pp:
            for c in range(4):
              cp.smem("psi out", pn + b * 4 * TY * Pp + c * TY * Pp, nrows * Pp,
                      pn, end)
        for c in range(3):
          cp.gmem("H out", (3 + c) * N + x * YZ + y0 * Z, nrows * Z, 6 * N)
          cp.gmem("E out", c * N + x * YZ + y0 * Z, nrows * Z, 6 * N)
        if Pp:
          for c in range(4):
            cp.gmem("psi out", c * PXY + (x * Y + y0) * Pp, nrows * Pp, 4 * PXY)
  return cp


def two_step(X, Y, Z, P, TY, SA, SB, seg_x):
  """Copies of yee_stream2_kernel for one launch (ring fills; its results
  are stored by the compute threads with 8-byte stores)."""
  Pp = r4(P)
  Yp = r4(Y)
  N, YZ, PXY = X * Y * Z, Y * Z, X * Y * Pp
  NR, NE, MT = TY + 3, TY + 4, r4(TY + 2) + 8
  a_e, a_h = 0, 3 * NE * Z
  a_p = a_h + 3 * NR * Z
  a_stage = a_p + 4 * NR * Pp
  b_c, b_m = 0, 3 * NR * Z
  b_stage = b_m + 3 * MT
  inter = 17 * NR * Z + 8 * NR * Pp
  nbytes = (SA * a_stage + SB * b_stage + inter) * 4 + (2 * SA + 2 * SB) * 8 + 16
  if nbytes > SMEM_BUDGET:
    return None
  ringB = SA * a_stage
  cp = Copies()
  for tile in range((Y + TY - 1) // TY):
    y0 = tile * TY
    ylo = max(y0 - 2, 0)
    e_hi, h_hi = min(y0 + TY + 2, Y), min(y0 + TY + 1, Y)
    clo = max(y0 - 1, 0)
    ma, mb = clo & ~3, min(r4(y0 + TY + 1), Yp)
    r0 = ylo - (y0 - 2)
    for seg in range((X + seg_x - 1) // seg_x):
      xs = seg * seg_x
      xe = min(X, xs + seg_x)
      a1 = max(xs - 2, 0)
      last1, lastA = min(xe, X - 1), min(xe + 1, X - 1)
      for xp in range(a1, lastA + 1):
        fullp = xp <= last1
        for slot in range(min(SA, 2)):
          st = slot * a_stage
          for c in range(3):
            cp.smem("E0", st + a_e + c * NE * Z + r0 * Z, (e_hi - ylo) * Z,
                    st + a_e + c * NE * Z, st + a_e + (c + 1) * NE * Z)
            if fullp:
              cp.smem("H0", st + a_h + c * NR * Z + r0 * Z, (h_hi - ylo) * Z,
                      st + a_h + c * NR * Z, st + a_h + (c + 1) * NR * Z)
          if fullp and Pp:
            for c in range(4):
              cp.smem("psi", st + a_p + c * NR * Pp + r0 * Pp, (h_hi - ylo) * Pp,
                      st + a_p + c * NR * Pp, st + a_p + (c + 1) * NR * Pp)
        for c in range(3):
          cp.gmem("E0", c * N + xp * YZ + ylo * Z, (e_hi - ylo) * Z, 6 * N)
          if fullp:
            cp.gmem("H0", (3 + c) * N + xp * YZ + ylo * Z, (h_hi - ylo) * Z, 6 * N)
        if fullp and Pp:
          for c in range(4):
            cp.gmem("psi", c * PXY + (xp * Y + ylo) * Pp, (h_hi - ylo) * Pp, 4 * PXY)
        if fullp:
          for slot in range(min(SB, 2)):
            st = ringB + slot * b_stage
            for c in range(3):
              cp.smem("cb", st + b_c + c * NR * Z + (clo - (y0 - 2)) * Z,
                      (h_hi - clo) * Z, st + b_c + c * NR * Z,
                      st + b_c + (c + 1) * NR * Z)
              cp.smem("mask", st + b_m + c * MT, mb - ma, st + b_m + c * MT,
                      st + b_m + (c + 1) * MT)
          for c in range(3):
            cp.gmem("cb", c * N + xp * YZ + clo * Z, (h_hi - clo) * Z, 3 * N)
            cp.gmem("mask", (xp * 3 + c) * Yp + ma, mb - ma, X * 3 * Yp)
  return cp


SHAPES = [(17, 5, 4), (24, 20, 16), (19, 33, 64), (40, 37, 32), (30, 21, 48),
          (9, 64, 12)]
PMLS = [0, 4, 8, 16]


@pytest.mark.parametrize("X,Y,Z", SHAPES)
@pytest.mark.parametrize("P", PMLS)
def test_one_step_copies_in_bounds_and_aligned(X, Y, Z, P):
  checked = 0
  for TY, S, seg_x in itertools.product((1, 2, 5, 14, 29), (2, 4), (1, 3, 8, X)):
    if TY > Y:
      continue
    for src in (None, (3, 0, 0, 2, Y, Z, 2), (0, min(3, Y - 1), 0, X, 1, Z, 6),
                (0, 0, 1, X, Y, 1, 4), (2, 1, 0, 5, min(2, Y - 1), Z, 2)):
      cp = one_step(X, Y, Z, P, TY, S, seg_x, src)
      if cp is None:
        continue
      assert not cp.bad, (X, Y, Z, P, TY, S, seg_x, src, cp.bad[:3])
      checked += cp.count
  assert checked > 0


@pytest.mark.parametrize("X,Y,Z", SHAPES)
@pytest.mark.parametrize("P", PMLS)
def test_two_step_copies_in_bounds_and_aligned(X, Y, Z, P):
  checked = 0
  for TY, SA, seg_x in itertools.product((1, 2, 6, 14), (2, 3), (1, 4, X)):
    if TY > Y:
      continue
    cp = two_step(X, Y, Z, P, TY, SA, SA, seg_x)
    if cp is None:
      continue
    assert not cp.bad, (X, Y, Z, P, TY, SA, seg_x, cp.bad[:3])
    checked += cp.count
  assert checked > 0


def test_model_flags_a_shape_the_host_refuses():
  """The host refuses the streamed kernels for zz % 4 != 0; the model shows
  why -- row copies of 6 floats are not whole 16-byte units."""
  cp = one_step(12, 10, 6, 0, 4, 2, 12)
  assert cp is not None and any(b[0] == "E" for b in cp.bad)
  cp2 = two_step(12, 10, 6, 0, 4, 2, 2, 12)
  assert cp2 is not None and cp2.bad
