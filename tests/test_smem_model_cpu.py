"""Shared-memory model of the streamed kernels' compute warps (CPU).

compute-sanitizer (memcheck, racecheck, initcheck) is closed on this machine.
This test restates `stream_tile` (`csrc/stream_kernel.cuh`, one step per
launch, with and without ring-carried source rows) and `stream2_tile`
(`csrc/stream2_kernel.cuh`, two steps per launch): their shared-memory
layouts, the producer's ring fills and bulk stores, and every shared-memory
load and store of the compute warps.  Each CTA's planes are replayed in one
legal order of the mbarrier protocol with a tag on every shared float that
names the data it holds -- field and component, time level (0: read from
HBM, 1: after the first step, 2: after the second), x-plane and y row; -1
means zero since the CTA started.  On a grid of shapes, PML widths, tiles,
ring depths, segments, source boxes and thread counts the test checks that

* every compute-warp access lies inside its region, and 64-bit accesses are
  8-byte aligned;
* every read sees exactly the field, component, level, plane and row the
  update needs, or a zero row outside the domain;
* no float is written by one thread and touched by another between two
  barriers;
* every float a bulk store reads was written for the plane it stores, both
  when the store may start (after the plane's E phase) and when it may
  still be reading (until the compute warps wait on it two planes later),
  and every output row of the launch is stored exactly once.

The one-step replay also takes the number of new-H buffers and of barriers
per plane as parameters, so that a change to that protocol is checked here
before it is made in the kernel.

It mirrors the kernels' index arithmetic line for line (the shared helpers
`h_pair` / `e_pair` follow the kernels' helpers of the same names); a
kernel change to that arithmetic must change this model with it.

The lean one-step kernel (`csrc/lean_kernel.cuh`) shares the streamed
kernel's producer and (with a third new-H buffer) its layout, so its replay
is the one-step replay with three new-H buffers, one barrier per plane and
the compute accesses swapped for the lean ones (`lean_items`, `lean_h`,
`lean_e`): one z-quad per thread, 128-bit accesses (checked 16-byte
aligned), interior and z-PML quads on separate warps.
"""

import itertools

import numpy as np
import pytest

SMEM_BUDGET = 220 * 1024       # tile selection budget of the host
SMEM_MAX = 227 * 1024 - 2048   # ring-carried source rows

# Tag = ((kind * 4 + level) * PLANE + plane) * ROW + y + 1.
ROW = 1 << 16
PLANE = 1 << 12
E, H, CB, MASK, PSI, SRC = 0, 3, 6, 9, 12, 16  # kinds: base + component
JSUM = 250     # + component: a source current after its sum
POISON = 255   # computed from a missing neighbour, must never be read


def r4(v):
  return (v + 3) & ~3


def tag(kind, level, plane, y):
  return ((np.asarray(kind) * 4 + level) * PLANE + plane) * ROW + np.asarray(y) + 1


def rows_tag(kind, level, plane, ylo, yhi, width):
  return np.repeat(tag(kind, level, plane, np.arange(ylo, yhi)), width)


class Smem:
  """Tagged shared memory of one CTA plus the access log of the current
  barrier interval."""

  def __init__(self, size):
    self.tag = np.full(size, -1, np.int64)
    self.bad = []
    self.reads = 0
    self.log = []  # (offsets, threads, is_write)

  def _where(self, what, off, lo, hi, width):
    """Checks bounds and alignment; returns the offsets, clipped into the
    buffer when they leave their region (the violation is recorded)."""
    off = np.asarray(off, np.int64)
    if off.size == 0:
      return off
    if off.min() < lo or off.max() + width > hi:
      self.bad.append((what, "bounds", int(off.min()), int(off.max()), lo, hi))
      off = np.clip(off, 0, len(self.tag) - width)
    if width == 2 and np.any(off % 2):
      self.bad.append((what, "align8", int(off[off % 2 != 0][0])))
    if width == 4 and np.any(off % 4):
      self.bad.append((what, "align16", int(off[off % 4 != 0][0])))
    return off

  def read(self, what, off, thr, expect, zero_ok, lo, hi, width=1):
    off = self._where(what, off, lo, hi, width)
    if off.size == 0:
      return
    thr = np.broadcast_to(np.asarray(thr, np.int64), off.shape).ravel()
    zero_ok = np.broadcast_to(np.asarray(zero_ok, bool), off.shape).ravel()
    expect = np.broadcast_to(np.asarray(expect, np.int64), off.shape).ravel()
    off = off.ravel()
    for w in range(width):
      t = self.tag[off + w]
      ok = (t == expect) | ((t == -1) & zero_ok)
      if not ok.all():
        i = int(np.argmin(ok))
        self.bad.append((what, "stale", int(off[i] + w), int(t[i]), int(expect[i])))
      self.log.append((off + w, thr, False))
    self.reads += off.size * width

  def write(self, what, off, thr, tags, lo, hi, width=1):
    off = self._where(what, off, lo, hi, width)
    if off.size == 0:
      return
    thr = np.broadcast_to(np.asarray(thr, np.int64), off.shape).ravel()
    tags = np.broadcast_to(np.asarray(tags, np.int64), off.shape).ravel()
    off = off.ravel()
    for w in range(width):
      self.tag[off + w] = tags
      self.log.append((off + w, thr, True))

  def end(self, what):
    """Closes a barrier interval: a float written by one thread and read or
    written by another inside it is a race."""
    if self.log:
      off = np.concatenate([o for o, _, _ in self.log])
      thr = np.concatenate([t for _, t, _ in self.log])
      wr = np.concatenate([np.full(o.shape, w) for o, _, w in self.log])
      sel = np.isin(off, np.unique(off[wr]))
      o, t = off[sel], thr[sel]
      order = np.lexsort((t, o))
      o, t = o[order], t[order]
      clash = (o[1:] == o[:-1]) & (t[1:] != t[:-1])
      if clash.any():
        i = int(np.argmax(clash))
        self.bad.append((what, "race", int(o[i]), int(t[i]), int(t[i + 1])))
    self.log = []

  def fill(self, off, tags):
    self.tag[off:off + len(tags)] = tags

  def stored(self, what, off, tags, mask=None):
    t = self.tag[off:off + len(tags)]
    ok = t == tags
    if mask is not None:
      ok |= ~mask
    if not ok.all():
      i = int(np.argmin(ok))
      self.bad.append((what, "store", off + i, int(t[i]), int(tags[i])))


class Ptr:
  """A shared-memory operand: base offset, component stride, the region it
  must stay in, and the tag its component c holds at row y."""

  def __init__(self, base, stride, lo, hi, T):
    self.base, self.stride, self.lo, self.hi, self.T = base, stride, lo, hi, T


def h_pair(sm, ph, thr, z0s, pz, Z, Y, Pp, ras, ys, Ep, E1p, Ho, Pin):
  """Shared-memory reads of the H updates of buffer rows `ras` (domain rows
  `ys`), z-pairs `z0s`, threads thr[row, pair]: E rows ra and ra + 1 and
  z + 2, E of plane x + 1 (E1p, or None at the last plane), old H, PML
  state comps 0 and 1."""
  ra, y = ras[:, None], ys[:, None]
  ie = ra * Z + z0s
  for c in range(3):
    sm.read(ph + ":E", Ep.base + c * Ep.stride + ie, thr, Ep.T(c, y), False,
            Ep.lo, Ep.hi, 2)
  up = y + 1 >= Y
  sm.read(ph + ":Ex y+1", Ep.base + ie + Z, thr, Ep.T(0, y + 1), up, Ep.lo, Ep.hi, 2)
  sm.read(ph + ":Ez y+1", Ep.base + 2 * Ep.stride + ie + Z, thr, Ep.T(2, y + 1), up,
          Ep.lo, Ep.hi, 2)
  zin = z0s + 2 < Z
  sm.read(ph + ":Ex z+1", (Ep.base + ie + 2)[:, zin], thr[:, zin], Ep.T(0, y),
          False, Ep.lo, Ep.hi)
  sm.read(ph + ":Ey z+1", (Ep.base + Ep.stride + ie + 2)[:, zin], thr[:, zin],
          Ep.T(1, y), False, Ep.lo, Ep.hi)
  if E1p is not None:
    for c in (1, 2):
      sm.read(ph + ":E x+1", E1p.base + c * E1p.stride + ie, thr, E1p.T(c, y), False,
              E1p.lo, E1p.hi, 2)
  for c in range(3):
    sm.read(ph + ":H", Ho.base + c * Ho.stride + ie, thr, Ho.T(c, y), False, Ho.lo,
            Ho.hi, 2)
  for q in range(2):
    on = pz[q] >= 0
    pi = ra * Pp + pz[q][on]
    for c in range(2):
      sm.read(ph + ":psi", Pin.base + c * Pin.stride + pi, thr[:, on], Pin.T(c, y),
              False, Pin.lo, Pin.hi)


def e_pair(sm, ph, thr, z0s, pz, Z, Pp, ras, ys, Hx, Hy, Hz, Hyp, Hzp, prev0, Eo,
           Cb, Pin):
  """Shared-memory reads of the E updates of buffer rows `ras` (domain rows
  `ys`): new H of the plane (rows ra, ra - 1, z - 1), new H y/z of plane
  x - 1 (zero when `prev0`), old E, coefficients, PML state comps 2, 3."""
  ra, y = ras[:, None], ys[:, None]
  ih = ra * Z + z0s
  for p in (Hx, Hy, Hz):
    sm.read(ph + ":H", p.base + ih, thr, p.T(0, y), False, p.lo, p.hi, 2)
  down = y - 1 < 0
  sm.read(ph + ":Hx y-1", Hx.base + ih - Z, thr, Hx.T(0, y - 1), down, Hx.lo, Hx.hi, 2)
  sm.read(ph + ":Hz y-1", Hz.base + ih - Z, thr, Hz.T(0, y - 1), down, Hz.lo, Hz.hi, 2)
  zin = z0s > 0
  sm.read(ph + ":Hx z-1", (Hx.base + ih - 1)[:, zin], thr[:, zin], Hx.T(0, y),
          False, Hx.lo, Hx.hi)
  sm.read(ph + ":Hy z-1", (Hy.base + ih - 1)[:, zin], thr[:, zin], Hy.T(0, y),
          False, Hy.lo, Hy.hi)
  for p in (Hyp, Hzp):
    sm.read(ph + ":H x-1", p.base + ih, thr, p.T(0, y), prev0, p.lo, p.hi, 2)
  for c in range(3):
    sm.read(ph + ":E", Eo.base + c * Eo.stride + ih, thr, Eo.T(c, y), False, Eo.lo,
            Eo.hi, 2)
    sm.read(ph + ":cb", Cb.base + c * Cb.stride + ih, thr, Cb.T(c, y), False, Cb.lo,
            Cb.hi, 2)
  for q in range(2):
    on = pz[q] >= 0
    pi = ra * Pp + pz[q][on]
    for c in range(2):
      sm.read(ph + ":psi", Pin.base + c * Pin.stride + pi, thr[:, on], Pin.T(c, y),
              False, Pin.lo, Pin.hi)


def phase_rows(lo, hi, y_of, keep, rpt, Zh, z0s):
  """Buffer rows [lo, hi) a phase updates (those `keep(y)` admits), their
  domain rows, and the thread of each (row, z-pair): row r belongs to the
  threads of row group r % rpt."""
  ras = np.array([r for r in range(lo, hi) if keep(y_of(r))], np.int64)
  ys = y_of(ras)
  thr = (ras % rpt)[:, None] * Zh + (z0s // 2)[None, :]
  return ras, ys, thr


def pml_columns(Z, plo, phi):
  z0s = np.arange(0, Z, 2)  # z0 of threads tid % Zh = 0 .. Zh-1
  pz = np.stack([np.where(z < plo, z, np.where(z >= Z - phi, z - (Z - phi) + plo, -1))
                 for z in (z0s, z0s + 1)])  # [q][pair]
  return z0s, pz


def lean_split(Z, plo, phi, esz):
  """The bank-conflict-free split mapping of ``lean_item`` applies."""
  return esz == 4 and Z == 64 and plo + phi <= 32


def lean_rows(Z, esz):
  """The row-major mapping of ``lean_item`` applies (binary16, or zz 32)."""
  return esz == 2 or Z == 32


def lean_items(Z, TY, plo, phi, esz=4):
  """Every compute thread's item in the lean kernels (``lean_item`` in
  csrc/lean_kernel.cuh) over TY + 1 buffer rows: thread ids, buffer row,
  quad start z0, z-PML state column, whether the quad is a z-PML quad, and
  the thread count.  Split mapping (FP32, zz 64, plo + phi <= 32): edge
  warps hold each row's quads [0, 8 - ph) and [16 - ph, 16) (ph = phi/4),
  interior warps quads [8 - ph, 16 - ph), 8 lanes per row.  Otherwise
  interior warps (quads between the slabs, row-major), then z-PML warps."""
  rows = TY + 1
  lq, pq, nq = plo // 4, phi // 4, Z // 4
  if lean_split(Z, plo, phi, esz):
    ne = (rows + 3) // 4
    thr = np.arange(32 * 2 * ne)
    w, j = thr >> 5, thr & 7
    edge = w < ne
    rH = 4 * np.where(edge, w, w - ne) + ((thr >> 3) & 3)
    q = np.where(edge, np.where(j < 8 - pq, j, j + 8), 8 - pq + j)
  elif lean_rows(Z, esz):
    thr = np.arange(32 * ((rows * nq + 31) // 32))
    rH, q = thr // nq, thr % nq
  else:
    QI, QP = (Z - plo - phi) // 4, (plo + phi) // 4
    nwi = (rows * QI + 31) // 32
    nwp = (rows * QP + 31) // 32
    thr = np.arange(32 * (nwi + nwp))
    pw = thr >= 32 * nwi
    i = np.where(pw, thr - 32 * nwi, thr)
    Qn = np.where(pw, QP, QI)
    rH = np.where(Qn > 0, i // np.maximum(Qn, 1), rows)
    qi = i - rH * Qn
    q = np.where(pw, np.where(qi < lq, qi, nq - QP + qi), lq + qi)
  pml = (q < lq) | (q >= nq - pq)
  col = 4 * np.where(q < lq, q, lq + q - (nq - pq))
  return thr, rH, 4 * q, np.where(pml, col, 0), pml, len(thr)


def lean_h(sm, it, Z, Y, Pp, y0, RH, ieH, ring_e, ring_e1, ring_h, ring_p,
           hcur, RHZ, pcur, po_hi, TY, x):
  """H-phase accesses of the lean kernel's items `it` (a boolean selection
  of lean_items) at plane x."""
  thr, rH, z0, col, pml = it
  y = y0 - 1 + rH
  ie = ieH
  Ep = ring_e
  for c in range(3):
    sm.read("LH:E", Ep.base + c * Ep.stride + ie, thr, Ep.T(c, y), False, Ep.lo,
            Ep.hi, 4)
  up = y + 1 >= Y
  sm.read("LH:Ex y+1", Ep.base + ie + Z, thr, Ep.T(0, y + 1), up, Ep.lo, Ep.hi, 4)
  sm.read("LH:Ez y+1", Ep.base + 2 * Ep.stride + ie + Z, thr, Ep.T(2, y + 1), up,
          Ep.lo, Ep.hi, 4)
  zin = z0 + 4 < Z
  sm.read("LH:Ex z+1", (Ep.base + ie + 4)[zin], thr[zin], Ep.T(0, y[zin]), False,
          Ep.lo, Ep.hi)
  sm.read("LH:Ey z+1", (Ep.base + Ep.stride + ie + 4)[zin], thr[zin],
          Ep.T(1, y[zin]), False, Ep.lo, Ep.hi)
  if ring_e1 is not None:
    for c in (1, 2):
      sm.read("LH:E x+1", ring_e1.base + c * ring_e1.stride + ie, thr,
              ring_e1.T(c, y), False, ring_e1.lo, ring_e1.hi, 4)
  for c in range(3):
    sm.read("LH:H", ring_h.base + c * ring_h.stride + ie, thr, ring_h.T(c, y), False,
            ring_h.lo, ring_h.hi, 4)
  pi = rH * Pp + col
  for c in range(2):
    sm.read("LH:psi", (ring_p.base + c * ring_p.stride + pi)[pml], thr[pml],
            ring_p.T(c, y[pml]), False, ring_p.lo, ring_p.hi, 4)
  for c in range(3):
    sm.write("LH out", hcur + c * RHZ + ie, thr, tag(H + c, 1, x, y), hcur,
             hcur + 3 * RHZ, 4)
  sel = pml & (rH > 0)
  po = (rH - 1) * Pp + col
  for c in range(2):
    sm.write("LH:psi out", (pcur + c * TY * Pp + po)[sel], thr[sel],
             tag(PSI + c, 1, x, y[sel]), pcur, po_hi, 4)


def lean_e(sm, it, Z, Pp, y0, RH, TY, hcur, hprev, RHZ, x, ring_e, Cs, c_lo, Ms,
           m_lo, MT, m_n, ring_p, ecur, pcur, po_hi):
  """E-phase accesses of the lean kernel's items `it` at plane x."""
  thr, rH, z0, col, pml = it
  y = y0 + rH
  ih = (rH + 1) * Z + z0
  ic = rH * Z + z0
  for c in range(3):
    sm.read("LE:H", hcur + c * RHZ + ih, thr, tag(H + c, 1, x, y), False, hcur,
            hcur + 3 * RHZ, 4)
  down = y - 1 < 0
  sm.read("LE:Hx y-1", hcur + ih - Z, thr, tag(H + 0, 1, x, y - 1), down, hcur,
          hcur + 3 * RHZ, 4)
  sm.read("LE:Hz y-1", hcur + 2 * RHZ + ih - Z, thr, tag(H + 2, 1, x, y - 1), down,
          hcur, hcur + 3 * RHZ, 4)
  zin = z0 > 0
  sm.read("LE:Hx z-1", (hcur + ih - 1)[zin], thr[zin], tag(H + 0, 1, x, y[zin]),
          False, hcur, hcur + 3 * RHZ)
  sm.read("LE:Hy z-1", (hcur + RHZ + ih - 1)[zin], thr[zin], tag(H + 1, 1, x, y[zin]),
          False, hcur, hcur + 3 * RHZ)
  for c in (1, 2):
    sm.read("LE:H x-1", hprev + c * RHZ + ih, thr, tag(H + c, 1, x - 1, y), x == 0,
            hprev, hprev + 3 * RHZ, 4)
  for c in range(3):
    sm.read("LE:E", ring_e.base + c * ring_e.stride + ih, thr, ring_e.T(c, y), False,
            ring_e.lo, ring_e.hi, 4)
    sm.read("LE:cb", Cs + c * TY * Z + ic, thr, tag(CB + c, 0, x, y), False, c_lo,
            c_lo + 3 * TY * Z, 4)
    sm.read("LE:mask", Ms + c * MT + rH, thr, tag(MASK + c, 0, x, y), False,
            m_lo + c * MT, m_lo + c * MT + m_n)
  pi = (rH + 1) * Pp + col
  for c in range(2):
    sm.read("LE:psi", (ring_p.base + (2 + c) * ring_p.stride + pi)[pml], thr[pml],
            ring_p.T(2 + c, y[pml]), False, ring_p.lo, ring_p.hi, 4)
  for c in range(3):
    sm.write("LE out", ecur + c * TY * Z + ic, thr, tag(E + c, 1, x, y), ecur,
             ecur + 3 * TY * Z, 4)
  po = rH * Pp + col
  for c in (2, 3):
    sm.write("LE:psi out", (pcur + c * TY * Pp + po)[pml], thr[pml],
             tag(PSI + c, 1, x, y[pml]), pcur, po_hi, 4)


def one_step_cta(X, Y, Z, plo, phi, TY, S, seg_x, tile, seg, ncomp, src, cover,
                 plant=None, hbuf=2, barriers=2, lean=False, esz=4):
  """Replays CTA (tile, seg) of yee_stream_kernel; returns its Smem or None
  when the host refuses the tile.  `cover[x, y]` counts the rows stored.
  `plant` puts a known mistake into the replay (for the tests that show the
  model catches it): "slot" reads plane x+1 from one ring slot too far,
  "moff" drops the absorber window offset.  `hbuf` (new-H buffers) and
  `barriers` (named barriers per plane) are 2 and 2 in the streamed kernel
  and 3 and 1 in the lean kernel, where the E phase of plane x shares its
  barrier interval with the H phase of plane x + 1.  The producer's
  stores of plane x are checked both right after its E phase and at the
  latest moment they may read, just before plane x + 2's wait on them."""
  P = plo + phi
  # PML state rows are whole 16-byte units: 4 FP32 or 8 binary16 values.
  Pp = r4(P) if esz == 4 else (P + 7) // 8 * 8
  Yp = r4(Y)
  RE, RH, MT = TY + 2, TY + 1, r4(TY) + 8
  e_off = 0
  h_off = e_off + 3 * RE * Z
  c_off = h_off + 3 * RH * Z
  m_off = c_off + 3 * TY * Z
  p_off = m_off + 3 * MT
  s_off = p_off + 4 * RH * Pp

  def smem_bytes(sw):
    # `esz` bytes per value (the absorber's FP32 windows are few).
    floats = S * (s_off + sw) + hbuf * 3 * RH * Z + 2 * 3 * TY * Z + 2 * 4 * TY * Pp
    return floats * esz + (2 * S + 2) * 8 + 16

  if smem_bytes(0) > SMEM_BUDGET:
    return None
  sw, sx0, sy0, sz0, snx, sny, snz, snc, srowf = 0, 0, 0, 0, 0, 0, 0, 0, 0
  if src is not None and not lean:
    sx0, sy0, sz0, snx, sny, snz, snc = src
    srowf = snc * 3 * snz
    rows = min(TY, sny)
    if srowf % 4 == 0 and smem_bytes(rows * srowf) <= SMEM_MAX:
      sw = rows * srowf
  SR = sw > 0
  stage = s_off + sw
  hn = S * stage
  en = hn + hbuf * 3 * RH * Z
  pn = en + 2 * 3 * TY * Z
  end = pn + 2 * 4 * TY * Pp
  RHZ, REZ = RH * Z, RE * Z
  sm = Smem(end)

  Zh = Z // 2
  rpt = ncomp // Zh
  litems = lean_items(Z, TY, plo, phi, esz) if lean else None
  y0 = tile * TY
  xs = seg * seg_x
  xe = min(X, xs + seg_x)
  x0 = xs - 1 if xs > 0 else 0
  xlast = min(xe, X - 1)
  ey_lo, ey_hi = max(y0 - 1, 0), min(y0 + TY + 1, Y)
  hy_hi = min(y0 + TY, Y)
  nrows = hy_hi - y0
  erow0 = ey_lo - (y0 - 1)
  ma, mb = y0 & ~3, min(r4(y0 + TY), Yp)
  moff = 0 if plant == "moff" else y0 - ma
  srow0 = max(y0, sy0)
  nsrow = min(min(y0 + TY, Y), sy0 + sny) - srow0
  z0s, pz = pml_columns(Z, plo, phi)
  src_kind = SRC + np.arange(srowf) // max(snz, 1)  # [column][component][z]

  def fill(xp, slot, fullp):
    st = slot * stage
    for c in range(3):
      sm.fill(st + e_off + c * REZ + erow0 * Z, rows_tag(E + c, 0, xp, ey_lo, ey_hi, Z))
    if not fullp:
      return
    for c in range(3):
      sm.fill(st + h_off + c * RHZ + erow0 * Z, rows_tag(H + c, 0, xp, ey_lo, hy_hi, Z))
      sm.fill(st + c_off + c * TY * Z, rows_tag(CB + c, 0, xp, y0, hy_hi, Z))
      sm.fill(st + m_off + c * MT, rows_tag(MASK + c, 0, xp, ma, mb, 1))
    for c in range(4 if Pp else 0):
      sm.fill(st + p_off + c * RH * Pp + erow0 * Pp,
              rows_tag(PSI + c, 0, xp, ey_lo, hy_hi, Pp))
    if SR and nsrow > 0 and sx0 <= xp < sx0 + snx:
      ys = np.arange(srow0, srow0 + nsrow)
      sm.fill(st + s_off, tag(src_kind[None, :], 0, xp, ys[:, None]).ravel())

  nfill = 0
  while nfill < S and x0 + nfill <= xlast:
    fill(x0 + nfill, nfill, x0 + nfill < xe)
    nfill += 1

  def stores(x, hcur, ecur, pcur):
    for c in range(3):
      sm.stored("H out", hcur + c * RHZ + Z, rows_tag(H + c, 1, x, y0, hy_hi, Z))
      sm.stored("E out", ecur + c * TY * Z, rows_tag(E + c, 1, x, y0, hy_hi, Z))
    if Pp:
      col = np.tile(np.arange(Pp) < P, nrows)
      for c in range(4):
        sm.stored("psi out", pcur + c * TY * Pp,
                  rows_tag(PSI + c, 1, x, y0, hy_hi, Pp), col)

  pending = {}  # plane index k -> its stores, checked again before k + 2
  slot, slot1 = 0, (1 if S > 1 else 0)
  for x in range(x0, xe):
    k = x - x0
    b = k & 1
    if k - 2 in pending:
      stores(*pending.pop(k - 2))
    st = slot * stage
    Es, E1 = st + e_off, slot1 * stage + e_off
    Hs, Cs, Ms, Ps = st + h_off, st + c_off, st + m_off + moff, st + p_off
    hcur, hprev = hn + (k % hbuf) * 3 * RHZ, hn + ((k - 1) % hbuf) * 3 * RHZ
    ecur, pcur = en + b * 3 * TY * Z, pn + b * 4 * TY * Pp
    po_hi = pcur + 4 * TY * Pp
    wr = x >= xs
    ring_e = Ptr(Es, REZ, Es, Es + 3 * REZ, lambda c, y, x=x: tag(E + c, 0, x, y))
    ring_e1 = (Ptr(E1, REZ, E1, E1 + 3 * REZ, lambda c, y, x=x: tag(E + c, 0, x + 1, y))
               if x + 1 < X else None)
    ring_h = Ptr(Hs, RHZ, Hs, Hs + 3 * RHZ, lambda c, y, x=x: tag(H + c, 0, x, y))
    ring_p = Ptr(Ps, RH * Pp, Ps, Ps + 4 * RH * Pp,
                 lambda c, y, x=x: tag(PSI + c, 0, x, y))

    # H phase: rows r = rt, rt + rpt, ... of threads rt < rpt.
    ras, ys, thr = phase_rows(0, RH, lambda r: y0 - 1 + r, lambda y: 0 <= y < Y, rpt,
                              Zh, z0s)
    if lean:
      yH = y0 - 1 + litems[1]
      sel = (litems[1] < RH) & (yH >= 0) & (yH < Y)
      it = tuple(v[sel] for v in litems[:5])
      lean_h(sm, it, Z, Y, Pp, y0, RH, it[1] * Z + it[2], ring_e, ring_e1, ring_h,
             ring_p, hcur, RHZ, pcur, po_hi, TY, x)
    elif len(ras):
      h_pair(sm, "H", thr, z0s, pz, Z, Y, Pp, ras, ys, ring_e, ring_e1, ring_h, ring_p)
      r, y = ras[:, None], ys[:, None]
      ie = r * Z + z0s
      pos = ras > 0
      for q in range(2):
        on = pz[q] >= 0
        po = (r[pos] - 1) * Pp + pz[q][on]
        for c in range(2):
          sm.write("H:psi out", pcur + c * TY * Pp + po, thr[pos][:, on],
                   tag(PSI + c, 1, x, y[pos]), pcur, po_hi)
      for c in range(3):
        sm.write("H out", hcur + c * RHZ + ie, thr, tag(H + c, 1, x, y), hcur,
                 hcur + 3 * RHZ, 2)

    src_plane = src is not None and sx0 <= x < sx0 + snx
    if SR and src_plane and nsrow > 0:
      # Cell t of the tile's box rows is summed by thread t % ncomp.
      t = np.arange(nsrow * snz)
      r = t // snz
      sv = st + s_off + r * srowf + (t - r * snz)
      for c in range(3):
        w3c = np.arange(snc) * 3 + c
        sm.read("J", (sv[:, None] + w3c * snz).ravel(), np.repeat(t % ncomp, snc),
                tag(SRC + w3c[None, :], 0, x, (srow0 + r)[:, None]).ravel(), False,
                st + s_off, st + stage)
        sm.write("J", sv + c * snz, t % ncomp, tag(JSUM + c, 0, x, srow0 + r),
                 st + s_off, st + stage)
    sm.end("H phase")

    if wr:
      hc = [Ptr(hcur + c * RHZ, 0, hcur, hcur + 3 * RHZ,
                lambda _, y, c=c, x=x: tag(H + c, 1, x, y)) for c in range(3)]
      hp = [Ptr(hprev + c * RHZ, 0, hprev, hprev + 3 * RHZ,
                lambda _, y, c=c, x=x: tag(H + c, 1, x - 1, y)) for c in range(3)]
      ring_cb = Ptr(Cs - Z, TY * Z, Cs, Cs + 3 * TY * Z,
                    lambda c, y, x=x: tag(CB + c, 0, x, y))
      ring_pe = Ptr(Ps + 2 * RH * Pp, RH * Pp, Ps, Ps + 4 * RH * Pp,
                    lambda c, y, x=x: tag(PSI + 2 + c, 0, x, y))
      ras, ys, thr = phase_rows(0, TY, lambda r: y0 + r, lambda y: y < Y, rpt, Zh, z0s)
      if lean:
        sel = (litems[1] < TY) & (y0 + litems[1] < Y)
        it = tuple(v[sel] for v in litems[:5])
        lean_e(sm, it, Z, Pp, y0, RH, TY, hcur, hprev, RHZ, x, ring_e, Cs, Cs, Ms,
               st + m_off, MT, mb - ma, ring_p, ecur, pcur, po_hi)
        ras = ys = np.zeros(0, np.int64)
        thr = np.zeros((0, len(z0s)), np.int64)
      else:
        e_pair(sm, "E", thr, z0s, pz, Z, Pp, ras + 1, ys, hc[0], hc[1], hc[2], hp[1],
               hp[2], x == 0, ring_e, ring_cb, ring_pe)
      r, y = ras[:, None], ys[:, None]
      for c in range(3):
        sm.read("E:mask", Ms + c * MT + ras, thr[:, 0], tag(MASK + c, 0, x, ys), False,
                st + m_off + c * MT, st + m_off + c * MT + (mb - ma))
      insrc = (ys >= sy0) & (ys < sy0 + sny)
      for q in range(2):
        on = pz[q] >= 0
        po = r * Pp + pz[q][on]
        for c in (2, 3):
          sm.write("E:psi out", pcur + c * TY * Pp + po, thr[:, on],
                   tag(PSI + c, 1, x, y), pcur, po_hi)
        if SR and src_plane and insrc.any():
          z = z0s + q
          cell = (z >= sz0) & (z < sz0 + snz)
          jv = st + s_off + (y[insrc] - srow0) * srowf + (z[cell] - sz0)
          for c in range(3):
            sm.read("E:J", jv + c * snz, thr[insrc][:, cell],
                    tag(JSUM + c, 0, x, y[insrc]), False, st + s_off, st + stage)
      ic = r * Z + z0s
      for c in range(3):
        sm.write("E out", ecur + c * TY * Z + ic, thr, tag(E + c, 1, x, y), ecur,
                 ecur + 3 * TY * Z, 2)
      if barriers == 2:
        sm.end("E phase")

    # Producer after done[slot]: bulk stores of plane x, then the refill.
    if wr:
      stores(x, hcur, ecur, pcur)
      pending[k] = (x, hcur, ecur, pcur)
      cover[x, y0:hy_hi] += 1
    if x0 + nfill <= xlast:
      fill(x0 + nfill, slot, x0 + nfill < xe)
      nfill += 1
    slot, slot1 = slot1, (slot1 + (2 if plant == "slot" else 1)) % S
  sm.end("last plane")
  for args in pending.values():
    stores(*args)
  return sm


def h_quad(sm, ph, it, Z, Y, Pp, ras, ys, Ep, E1p, Ho, Pin):
  """Shared-memory reads of lean H updates (quads): items ``it`` (thread,
  quad start, PML column, PML warp) at buffer rows ``ras`` (domain rows
  ``ys``): E rows ra and ra + 1 and z + 4, E of plane x + 1, old H, PML
  state comps 0 and 1."""
  thr, z0, col, pml = it
  ie = ras * Z + z0
  for c in range(3):
    sm.read(ph + ":E", Ep.base + c * Ep.stride + ie, thr, Ep.T(c, ys), False,
            Ep.lo, Ep.hi, 4)
  up = ys + 1 >= Y
  sm.read(ph + ":Ex y+1", Ep.base + ie + Z, thr, Ep.T(0, ys + 1), up, Ep.lo, Ep.hi, 4)
  sm.read(ph + ":Ez y+1", Ep.base + 2 * Ep.stride + ie + Z, thr, Ep.T(2, ys + 1), up,
          Ep.lo, Ep.hi, 4)
  zin = z0 + 4 < Z
  sm.read(ph + ":Ex z+1", (Ep.base + ie + 4)[zin], thr[zin], Ep.T(0, ys[zin]),
          False, Ep.lo, Ep.hi)
  sm.read(ph + ":Ey z+1", (Ep.base + Ep.stride + ie + 4)[zin], thr[zin],
          Ep.T(1, ys[zin]), False, Ep.lo, Ep.hi)
  if E1p is not None:
    for c in (1, 2):
      sm.read(ph + ":E x+1", E1p.base + c * E1p.stride + ie, thr, E1p.T(c, ys), False,
              E1p.lo, E1p.hi, 4)
  for c in range(3):
    sm.read(ph + ":H", Ho.base + c * Ho.stride + ie, thr, Ho.T(c, ys), False, Ho.lo,
            Ho.hi, 4)
  pi = ras * Pp + col
  for c in range(2):
    sm.read(ph + ":psi", (Pin.base + c * Pin.stride + pi)[pml], thr[pml],
            Pin.T(c, ys[pml]), False, Pin.lo, Pin.hi, 4)


def e_quad(sm, ph, it, Z, Pp, ras, ys, Hx, Hy, Hz, Hyp, Hzp, prev0, Eo, Cb, Pin):
  """Shared-memory reads of lean E updates (quads) at buffer rows ``ras``:
  new H of the plane (rows ra, ra - 1, z - 1), new H y/z of plane x - 1
  (zero when ``prev0``), old E, coefficients, PML state comps 2, 3."""
  thr, z0, col, pml = it
  ih = ras * Z + z0
  for p in (Hx, Hy, Hz):
    sm.read(ph + ":H", p.base + ih, thr, p.T(0, ys), False, p.lo, p.hi, 4)
  down = ys - 1 < 0
  sm.read(ph + ":Hx y-1", Hx.base + ih - Z, thr, Hx.T(0, ys - 1), down, Hx.lo,
          Hx.hi, 4)
  sm.read(ph + ":Hz y-1", Hz.base + ih - Z, thr, Hz.T(0, ys - 1), down, Hz.lo,
          Hz.hi, 4)
  zin = z0 > 0
  sm.read(ph + ":Hx z-1", (Hx.base + ih - 1)[zin], thr[zin], Hx.T(0, ys[zin]),
          False, Hx.lo, Hx.hi)
  sm.read(ph + ":Hy z-1", (Hy.base + ih - 1)[zin], thr[zin], Hy.T(0, ys[zin]),
          False, Hy.lo, Hy.hi)
  for p in (Hyp, Hzp):
    sm.read(ph + ":H x-1", p.base + ih, thr, p.T(0, ys), prev0, p.lo, p.hi, 4)
  for c in range(3):
    sm.read(ph + ":E", Eo.base + c * Eo.stride + ih, thr, Eo.T(c, ys), False, Eo.lo,
            Eo.hi, 4)
    sm.read(ph + ":cb", Cb.base + c * Cb.stride + ih, thr, Cb.T(c, ys), False, Cb.lo,
            Cb.hi, 4)
  pi = ras * Pp + col
  for c in range(2):
    sm.read(ph + ":psi", (Pin.base + c * Pin.stride + pi)[pml], thr[pml],
            Pin.T(c, ys[pml]), False, Pin.lo, Pin.hi, 4)


def two_step_cta(X, Y, Z, plo, phi, TY, SA, SB, seg_x, tile, seg, ncomp, cover,
                 lean=False, esz=4):
  """Replays CTA (tile, seg) of yee_stream2_kernel; returns its Smem or None
  when the host refuses the tile.  Level-2 results go straight to global
  memory; `cover[level - 1 of the phase, x, y]` counts the rows stored."""
  P = plo + phi
  Pp = r4(P) if esz == 4 else (P + 7) // 8 * 8
  Yp = r4(Y)
  NR, NE, MT = TY + 3, TY + 4, r4(TY + 2) + 8
  NRZ, NEZ, NRP = NR * Z, NE * Z, NR * Pp
  a_e, a_h = 0, 3 * NEZ
  a_p = a_h + 3 * NRZ
  a_stage = a_p + 4 * NRP
  b_c, b_m = 0, 3 * NRZ
  b_stage = b_m + 3 * MT
  inter = 17 * NRZ + 8 * NRP
  if (SA * a_stage + SB * b_stage + inter) * 4 + (2 * SA + 2 * SB) * 8 + 16 > SMEM_BUDGET:
    return None
  ringB = SA * a_stage
  H1 = ringB + SB * b_stage
  E1 = H1 + 6 * NRZ
  H2x = E1 + 6 * NRZ
  H2yz = H2x + NRZ
  P1 = H2yz + 4 * NRZ
  sm = Smem(P1 + 8 * NRP)

  Zh = Z // 2
  rpt = ncomp // Zh
  y0 = tile * TY
  xs = seg * seg_x
  xe = min(X, xs + seg_x)
  a1, a2 = max(xs - 2, 0), max(xs - 1, 0)
  last1, lastA = min(xe, X - 1), min(xe + 1, X - 1)
  ylo = max(y0 - 2, 0)
  e_hi, h_hi = min(y0 + TY + 2, Y), min(y0 + TY + 1, Y)
  clo = max(y0 - 1, 0)
  ma, mb = clo & ~3, min(r4(y0 + TY + 1), Yp)
  r0 = ylo - (y0 - 2)
  z0s, pz = pml_columns(Z, plo, phi)

  def fillA(xp, slot):
    st = slot * a_stage
    for c in range(3):
      sm.fill(st + a_e + c * NEZ + r0 * Z, rows_tag(E + c, 0, xp, ylo, e_hi, Z))
    if xp > last1:
      return
    for c in range(3):
      sm.fill(st + a_h + c * NRZ + r0 * Z, rows_tag(H + c, 0, xp, ylo, h_hi, Z))
    for c in range(4 if Pp else 0):
      sm.fill(st + a_p + c * NRP + r0 * Pp, rows_tag(PSI + c, 0, xp, ylo, h_hi, Pp))

  def fillB(xp, slot):
    st = ringB + slot * b_stage
    for c in range(3):
      sm.fill(st + b_c + c * NRZ + (clo - (y0 - 2)) * Z,
              rows_tag(CB + c, 0, xp, clo, h_hi, Z))
      sm.fill(st + b_m + c * MT, rows_tag(MASK + c, 0, xp, ma, mb, 1))

  nA = nB = 0
  while nA < SA and a1 + nA <= lastA:
    fillA(a1 + nA, nA)
    nA += 1
  while nB < SB and a1 + nB <= last1:
    fillB(a1 + nB, nB)
    nB += 1
  pA = pB = 0  # the producer's ring positions
  sA, sA1 = 0, (1 if SA > 1 else 0)
  sB = sBm = 0

  def ydom(ra):
    return y0 - 2 + ra

  def buf(base, stride, n, kind, level, plane):
    return Ptr(base, stride, base, base + n,
               lambda c, y: tag(kind + c, level, plane, y))

  if lean:  # one (buffer row, quad) item per thread over the NR rows
    lthr, lra, lz0, lcol, lpml, _ = lean_items(Z, NR - 1, plo, phi, esz)
    lys = y0 - 2 + lra

  def items(lo, hi, keep):
    """Lean items whose buffer row is in [lo, hi) and whose domain row
    `keep` admits: (thread, quad start, PML column, PML warp), rows, ys."""
    sel = (lra >= lo) & (lra < hi) & keep(lys)
    return (lthr[sel], lz0[sel], lcol[sel], lpml[sel]), lra[sel], lys[sel]

  for x in range(a1, xe + 1):
    l1, l2, st2 = x <= last1, x - 1 >= a2, x - 1 >= xs
    b = x & 1
    As, A1s = sA * a_stage, sA1 * a_stage
    Bs, Bm = ringB + sB * b_stage, ringB + sBm * b_stage
    h1c, h1p = H1 + b * 3 * NRZ, H1 + (b ^ 1) * 3 * NRZ
    e1c, e1p = E1 + b * 3 * NRZ, E1 + (b ^ 1) * 3 * NRZ
    p1c, p1p = P1 + b * 4 * NRP, P1 + (b ^ 1) * 4 * NRP
    h2yz, h2yzp = H2yz + (b ^ 1) * 2 * NRZ, H2yz + b * 2 * NRZ

    # Level 1, H(x), rows y0-2 .. y0+TY (same interval as the previous
    # plane's level-2 E phase: no barrier between them).
    if l1:
      a_rng = (As, As + a_stage)
      Ep = Ptr(As + a_e, NEZ, *a_rng, lambda c, y, x=x: tag(E + c, 0, x, y))
      E1p = (Ptr(A1s + a_e, NEZ, A1s, A1s + a_stage,
                 lambda c, y, x=x: tag(E + c, 0, x + 1, y)) if x + 1 < X else None)
      Ho = Ptr(As + a_h, NRZ, *a_rng, lambda c, y, x=x: tag(H + c, 0, x, y))
      Pin = Ptr(As + a_p, NRP, *a_rng, lambda c, y, x=x: tag(PSI + c, 0, x, y))
      ras, ys, thr = phase_rows(0, NR, ydom, lambda y: 0 <= y < Y, rpt, Zh, z0s)
      if lean:
        it, ra_, y_ = items(0, NR, lambda y: (y >= 0) & (y < Y))
        h_quad(sm, "L1 H", it, Z, Y, Pp, ra_, y_, Ep, E1p, Ho, Pin)
        ie = ra_ * Z + it[1]
        for c in range(3):
          sm.write("L1 H out", h1c + c * NRZ + ie, it[0], tag(H + c, 1, x, y_), h1c,
                   h1c + 3 * NRZ, 4)
        m = it[3]
        for c in range(2):
          sm.write("L1 H psi", (p1c + c * NRP + ra_ * Pp + it[2])[m], it[0][m],
                   tag(PSI + c, 1, x, y_[m]), p1c, p1c + 4 * NRP, 4)
        ras = ras[:0]
      if len(ras):
        h_pair(sm, "L1 H", thr, z0s, pz, Z, Y, Pp, ras, ys, Ep, E1p, Ho, Pin)
        ra, y = ras[:, None], ys[:, None]
        ie = ra * Z + z0s
        for c in range(3):
          sm.write("L1 H out", h1c + c * NRZ + ie, thr, tag(H + c, 1, x, y), h1c,
                   h1c + 3 * NRZ, 2)
        for q in range(2):
          on = pz[q] >= 0
          for c in range(2):
            sm.write("L1 H psi", p1c + c * NRP + ra * Pp + pz[q][on], thr[:, on],
                     tag(PSI + c, 1, x, y), p1c, p1c + 4 * NRP)
    sm.end("level-2 E + level-1 H")
    if l1:
      # Plane a1 > 0 has no level-1 H of plane a1 - 1: its level-1 E is
      # computed from zeros and must never be read.
      poison = x == a1 and a1 > 0
      Ms = Bs + b_m + (y0 - 2 - ma)
      hc = [buf(h1c + c * NRZ, 0, 3 * NRZ - c * NRZ, H + c, 1, x) for c in range(3)]
      hp = [buf(h1p + c * NRZ, 0, 3 * NRZ - c * NRZ, H + c, 1, x - 1) for c in range(3)]
      Eo = Ptr(As + a_e, NEZ, As, As + a_stage, lambda c, y, x=x: tag(E + c, 0, x, y))
      Cb = Ptr(Bs + b_c, NRZ, Bs, Bs + b_stage, lambda c, y, x=x: tag(CB + c, 0, x, y))
      Pe = Ptr(As + a_p + 2 * NRP, NRP, As, As + a_stage,
               lambda c, y, x=x: tag(PSI + 2 + c, 0, x, y))
      ras, ys, thr = phase_rows(1, NR, ydom, lambda y: 0 <= y < Y, rpt, Zh, z0s)
      if lean:
        it, ra_, y_ = items(1, NR, lambda y: (y >= 0) & (y < Y))
        for c in range(3):
          sm.read("L1 E:mask", Ms + c * MT + ra_, it[0], tag(MASK + c, 0, x, y_),
                  False, Bs + b_m + c * MT, Bs + b_m + c * MT + (mb - ma))
        e_quad(sm, "L1 E", it, Z, Pp, ra_, y_, hc[0], hc[1], hc[2], hp[1], hp[2],
               x == 0 or poison, Eo, Cb, Pe)
        ie = ra_ * Z + it[1]
        for c in range(3):
          out = tag(POISON, 1, x, y_) if poison else tag(E + c, 1, x, y_)
          sm.write("L1 E out", e1c + c * NRZ + ie, it[0], out, e1c, e1c + 3 * NRZ, 4)
        m = it[3]
        for c in (2, 3):
          sm.write("L1 E psi", (p1c + c * NRP + ra_ * Pp + it[2])[m], it[0][m],
                   tag(PSI + c, 1, x, y_[m]), p1c, p1c + 4 * NRP, 4)
        ras = ras[:0]
      if len(ras):
        for c in range(3):
          sm.read("L1 E:mask", Ms + c * MT + ras, thr[:, 0], tag(MASK + c, 0, x, ys),
                  False, Bs + b_m + c * MT, Bs + b_m + c * MT + (mb - ma))
        e_pair(sm, "L1 E", thr, z0s, pz, Z, Pp, ras, ys, hc[0], hc[1], hc[2], hp[1],
               hp[2], x == 0 or poison, Eo, Cb, Pe)
        ra, y = ras[:, None], ys[:, None]
        ie = ra * Z + z0s
        for c in range(3):
          out = tag(POISON, 1, x, y) if poison else tag(E + c, 1, x, y)
          sm.write("L1 E out", e1c + c * NRZ + ie, thr, out, e1c, e1c + 3 * NRZ, 2)
        for q in range(2):
          on = pz[q] >= 0
          for c in (2, 3):
            sm.write("L1 E psi", p1c + c * NRP + ra * Pp + pz[q][on], thr[:, on],
                     tag(PSI + c, 1, x, y), p1c, p1c + 4 * NRP)
      # doneA[plane x]: the producer refills the slot.
      if a1 + nA <= lastA:
        fillA(a1 + nA, pA)
        nA += 1
      pA = (pA + 1) % SA
    sm.end("level-1 E")

    xm = x - 1
    if l2:
      Ep = buf(e1p, NRZ, 3 * NRZ, E, 1, xm)
      E1p = buf(e1c, NRZ, 3 * NRZ, E, 1, x) if x < X else None
      Ho = buf(h1p, NRZ, 3 * NRZ, H, 1, xm)
      Pin = buf(p1p, NRP, 4 * NRP, PSI, 1, xm)
      ras, ys, thr = phase_rows(1, NR - 1, ydom, lambda y: 0 <= y < Y, rpt, Zh, z0s)
      if lean:
        it, ra_, y_ = items(1, NR - 1, lambda y: (y >= 0) & (y < Y))
        h_quad(sm, "L2 H", it, Z, Y, Pp, ra_, y_, Ep, E1p, Ho, Pin)
        ie = ra_ * Z + it[1]
        sm.write("L2 Hx", H2x + ie, it[0], tag(H, 2, xm, y_), H2x, H2x + NRZ, 4)
        for c in (1, 2):
          sm.write("L2 Hyz", h2yz + (c - 1) * NRZ + ie, it[0], tag(H + c, 2, xm, y_),
                   h2yz, h2yz + 2 * NRZ, 4)
        if st2:
          cover[0, xm, y_[ra_ >= 2]] += 1
        ras = ras[:0]
      if len(ras):
        h_pair(sm, "L2 H", thr, z0s, pz, Z, Y, Pp, ras, ys, Ep, E1p, Ho, Pin)
        ra, y = ras[:, None], ys[:, None]
        ie = ra * Z + z0s
        sm.write("L2 Hx", H2x + ie, thr, tag(H, 2, xm, y), H2x, H2x + NRZ, 2)
        for c in (1, 2):
          sm.write("L2 Hyz", h2yz + (c - 1) * NRZ + ie, thr, tag(H + c, 2, xm, y),
                   h2yz, h2yz + 2 * NRZ, 2)
        if st2:
          cover[0, xm, ys[ras >= 2]] += 1
    sm.end("level-2 H")

    if st2:
      Ms = Bm + b_m + (y0 - 2 - ma)
      hx = buf(H2x, 0, NRZ, H, 2, xm)
      hy = buf(h2yz, 0, 2 * NRZ, H + 1, 2, xm)
      hz = buf(h2yz + NRZ, 0, NRZ, H + 2, 2, xm)
      hyp = buf(h2yzp, 0, 2 * NRZ, H + 1, 2, xm - 1)
      hzp = buf(h2yzp + NRZ, 0, NRZ, H + 2, 2, xm - 1)
      Eo = buf(e1p, NRZ, 3 * NRZ, E, 1, xm)
      Cb = Ptr(Bm + b_c, NRZ, Bm, Bm + b_stage, lambda c, y: tag(CB + c, 0, xm, y))
      Pe = Ptr(p1p + 2 * NRP, NRP, p1p, p1p + 4 * NRP,
               lambda c, y: tag(PSI + 2 + c, 1, xm, y))
      ras, ys, thr = phase_rows(2, NR - 1, ydom, lambda y: y < Y, rpt, Zh, z0s)
      if lean:
        it, ra_, y_ = items(2, NR - 1, lambda y: y < Y)
        for c in range(3):
          sm.read("L2 E:mask", Ms + c * MT + ra_, it[0], tag(MASK + c, 0, xm, y_),
                  False, Bm + b_m + c * MT, Bm + b_m + c * MT + (mb - ma))
        e_quad(sm, "L2 E", it, Z, Pp, ra_, y_, hx, hy, hz, hyp, hzp, xm == 0, Eo, Cb,
               Pe)
        cover[1, xm, y_] += 1
        ras = ras[:0]
      if len(ras):
        for c in range(3):
          sm.read("L2 E:mask", Ms + c * MT + ras, thr[:, 0], tag(MASK + c, 0, xm, ys),
                  False, Bm + b_m + c * MT, Bm + b_m + c * MT + (mb - ma))
        e_pair(sm, "L2 E", thr, z0s, pz, Z, Pp, ras, ys, hx, hy, hz, hyp, hzp, xm == 0,
               Eo, Cb, Pe)
        cover[1, xm, ys] += 1
    if x > a1 and x - 1 <= last1:
      # doneB[plane x - 1]: the producer refills the slot.
      if a1 + nB <= last1:
        fillB(a1 + nB, pB)
        nB += 1
      pB = (pB + 1) % SB
    if l1:
      sA, sA1 = sA1, (sA1 + 1) % SA
      sBm, sB = sB, (sB + 1) % SB
    else:
      sBm = sB
  sm.end("level-2 E")
  return sm


def run_grid(cta, X, Y, TY, seg_x, cover_shape):
  """Runs every CTA of one launch; returns (reads, violations, cover) or
  None when the host refuses the tile."""
  reads, bad = 0, []
  cover = np.zeros(cover_shape, np.int64)
  for tile in range((Y + TY - 1) // TY):
    for seg in range((X + seg_x - 1) // seg_x):
      sm = cta(tile, seg, cover)
      if sm is None:
        return None
      reads += sm.reads
      bad += [(tile, seg) + b for b in sm.bad]
  return reads, bad, cover


def one_step(X, Y, Z, plo, phi, TY, S, seg_x, ncomp, src, plant=None, hbuf=2,
             barriers=2, lean=False, esz=4):
  def cta(tile, seg, cover):
    return one_step_cta(X, Y, Z, plo, phi, TY, S, seg_x, tile, seg, ncomp, src,
                        cover, plant, hbuf, barriers, lean, esz)
  return run_grid(cta, X, Y, TY, seg_x, (X, Y))


def two_step(X, Y, Z, plo, phi, TY, SA, seg_x, ncomp, lean=False, esz=4):
  def cta(tile, seg, cover):
    return two_step_cta(X, Y, Z, plo, phi, TY, SA, SA, seg_x, tile, seg, ncomp, cover,
                        lean, esz)
  return run_grid(cta, X, Y, TY, seg_x, (2, X, Y))


def host_ncomp(Z, TY):
  """Compute threads of the one-step kernel the host launches by default."""
  rpt = max(1, (512 - 32) // (Z // 2))
  return ((Z // 2) * min(rpt, TY + 1) + 31) // 32 * 32


def host_ncomp2(Z, TY):
  """Compute threads of the two-step kernel (generic body)."""
  rows = min((576 - 32) // (Z // 2), TY + 3)
  return ((Z // 2) * rows + 31) // 32 * 32


def min_ncomp(Z):
  """Fewest whole warps that cover one z column."""
  return max(32, (Z // 2 + 31) // 32 * 32)


SHAPES = [(7, 5, 4), (9, 20, 16), (6, 13, 64), (8, 11, 32), (5, 9, 48)]
SHAPES2 = [(7, 5, 4), (9, 14, 16), (6, 13, 64), (8, 11, 32), (5, 9, 48)]
PMLS = [(0, 0), (2, 2), (1, 3)]
SOURCES = [None, (2, 0, 0, 2, None, None, 2), (0, 3, 0, None, 1, None, 6),
           (0, 0, 1, None, None, 1, 4), (1, 1, 0, 3, 2, None, 2),
           (1, 2, 2, 2, 3, 2, 2)]


def source_box(i, X, Y, Z):
  """Source box i of SOURCES fitted to the domain (None entries: full
  extent)."""
  s = SOURCES[i % len(SOURCES)]
  if s is None:
    return None
  sx0, sy0, sz0, snx, sny, snz, snc = s
  sy0 = min(sy0, Y - 1)
  snx = X - sx0 if snx is None else min(snx, X - sx0)
  sny = Y - sy0 if sny is None else min(sny, Y - sy0)
  snz = Z - sz0 if snz is None else min(snz, Z - sz0)
  return (sx0, sy0, sz0, snx, sny, snz, snc)


@pytest.mark.parametrize("X,Y,Z", SHAPES)
@pytest.mark.parametrize("plo,phi", PMLS)
def test_one_step_compute_accesses(X, Y, Z, plo, phi):
  """Every (tile height, ring depth, segment) combination, cycling through
  the source boxes and the two thread counts (the host's default and the
  fewest warps that cover one z column)."""
  checked = 0
  combos = itertools.product((1, 2, 5, 14), (2, 4), (3, X))
  for i, (TY, S, seg_x) in enumerate(combos):
    if TY > Y:
      continue
    ncomp = host_ncomp(Z, TY) if i % 2 == 0 else min_ncomp(Z)
    src = source_box(i + plo, X, Y, Z)
    res = one_step(X, Y, Z, plo, phi, TY, S, seg_x, ncomp, src)
    if res is None:
      continue
    reads, bad, cover = res
    assert not bad, (X, Y, Z, plo, phi, TY, S, seg_x, ncomp, src, bad[:3])
    assert (cover == 1).all(), (TY, S, seg_x)
    checked += reads
  assert checked > 0


@pytest.mark.parametrize("X,Y,Z", SHAPES2)
@pytest.mark.parametrize("plo,phi", PMLS)
def test_two_step_compute_accesses(X, Y, Z, plo, phi):
  """Every (tile height, ring depth, segment) combination of the two-step
  kernel, alternating the two thread counts; one-plane segments put both
  halo planes of every segment inside the domain."""
  checked = 0
  combos = itertools.product((1, 6, 14), (2, 3), (1, X))
  for i, (TY, SA, seg_x) in enumerate(combos):
    if TY > Y:
      continue
    ncomp = host_ncomp2(Z, TY) if i % 2 == 0 else min_ncomp(Z)
    res = two_step(X, Y, Z, plo, phi, TY, SA, seg_x, ncomp)
    if res is None:
      continue
    reads, bad, cover = res
    assert not bad, (X, Y, Z, plo, phi, TY, SA, seg_x, ncomp, bad[:3])
    assert (cover == 1).all(), (TY, SA, seg_x)
    checked += reads
  assert checked > 0


@pytest.mark.parametrize("plant,what", [("slot", "H:E x+1"), ("moff", "E:mask")])
def test_model_flags_a_planted_mistake(plant, what):
  """A plane read from the wrong ring slot, and an absorber value read from
  the wrong y row, are both reported as stale reads."""
  args = (9, 20, 16, 2, 2, 5, 3, 3, 32, (2, 0, 0, 2, 20, 16, 2))
  assert one_step(*args)[1] == []
  res = one_step(*args, plant=plant)
  assert any(b[2] == what and b[3] == "stale" for b in res[1])


def test_model_flags_a_race():
  """A float written by one thread and read by another inside one barrier
  interval is reported."""
  sm = Smem(16)
  sm.write("w", [4], 0, 1, 0, 16)
  sm.read("r", [4], 1, 1, False, 0, 16)
  sm.end("phase")
  assert any(b[1] == "race" for b in sm.bad)


def test_one_barrier_protocol_needs_three_h_buffers():
  """A candidate change to the one-step kernel, checked before it is made.
  Dropping the barrier after the E phase lets plane x's E phase overlap
  plane x + 1's H phase.  With two new-H buffers that overlap is a race
  (H(x + 1) overwrites H(x - 1), which E(x) still reads).  With three
  buffers the replay is clean, including the producer's delayed stores.
  The third buffer fits the production tile (zz 64, tile_y 14, 4 ring
  stages, 16-cell PML) within the host's shared-memory budget."""
  cases = [(9, 20, 16, 2, 2, 5, 3, 3, 32, (2, 0, 0, 2, 20, 16, 2)),
           (8, 11, 32, 1, 3, 5, 4, 8, 192, (0, 0, 1, 8, 11, 1, 4)),
           (6, 13, 64, 2, 2, 14, 4, 6, 480, None)]
  for c in cases:
    assert one_step(*c, hbuf=2, barriers=2)[1] == []
    assert one_step(*c, hbuf=3, barriers=1)[1] == []
    assert any(b[3] == "race" for b in one_step(*c, hbuf=2, barriers=1)[1])
  RE, RH, TY, Z, Pp, S = 16, 15, 14, 64, 16, 4
  stage = 3 * RE * Z + 3 * RH * Z + 3 * TY * Z + 3 * (r4(TY) + 8) + 4 * RH * Pp
  for hbuf, fits in ((2, True), (3, True), (4, False)):
    floats = S * stage + hbuf * 3 * RH * Z + 2 * 3 * TY * Z + 2 * 4 * TY * Pp
    assert (floats * 4 + (2 * S + 2) * 8 + 16 <= SMEM_BUDGET) == fits


def test_random_shapes():
  """Seeded random launches beyond the grid above: any zz that is a
  multiple of 4 up to 64, tile heights to 29, ring depths 2-8, uneven PML
  slabs, both thread counts, every source box; one- and two-step."""
  import random
  rng = random.Random(1)
  done = 0
  while done < 30:
    Z = rng.choice(range(4, 68, 4))
    X, Y = rng.randint(2, 9), rng.randint(1, 40)
    plo, phi = rng.randint(0, min(4, Z // 4)), rng.randint(0, min(4, Z // 4))
    TY, S, seg = rng.randint(1, min(Y, 29)), rng.randint(2, 8), rng.randint(1, X)
    nc = rng.choice([host_ncomp(Z, TY), min_ncomp(Z)])
    src = source_box(rng.randint(0, 5), X, Y, Z)
    res = one_step(X, Y, Z, plo, phi, TY, S, seg, nc, src)
    if res is not None:
      assert not res[1] and (res[2] == 1).all(), (X, Y, Z, plo, phi, TY, S, seg,
                                                   nc, src, res[1][:2])
      done += 1
    TY2 = rng.randint(1, min(Y, 14))
    nc2 = rng.choice([host_ncomp2(Z, TY2), min_ncomp(Z)])
    res = two_step(X, Y, Z, plo, phi, TY2, rng.randint(2, 3), seg, nc2)
    if res is not None:
      assert not res[1] and (res[2] == 1).all(), (X, Y, Z, plo, phi, TY2, seg,
                                                   nc2, res[1][:2])


# The lean kernel's new-H buffers and barriers per plane.
LEAN_PROTOCOL = dict(hbuf=3, barriers=1)

# Tall tiles of the binary16 lean kernel (PJZ_LEAN_SHAPES_F16).
LEAN_F16_ONLY = {(64, 28)}

LEAN_CASES = [(5, 30, 64, 14), (4, 41, 48, 19), (3, 61, 32, 29), (6, 9, 16, 5),
              (4, 13, 24, 3), (3, 61, 64, 28)]


@pytest.mark.parametrize("esz", [4, 2])
@pytest.mark.parametrize("X,Y,Z,TY", LEAN_CASES)
@pytest.mark.parametrize("plo,phi", [(0, 0), (4, 4), (8, 8), (4, 8), (12, 4)])
def test_lean_compute_accesses(X, Y, Z, TY, plo, phi, esz):
  """The lean kernel's items (z-quads, interior and PML warps) over ring
  depths and segments, with a tile boundary inside the domain and a ragged
  last tile: in bounds, quad-aligned (16 bytes for FP32, 8 for binary16
  storage, whose PML state rows are 8 values), reading exactly the data
  each update needs, race-free between barriers, every row stored once."""
  if plo + phi > Z:
    pytest.skip("slabs wider than the domain")
  if (Z, TY) in LEAN_F16_ONLY and esz != 2:
    pytest.skip("a binary16-only shape")
  checked = 0
  for S, seg_x in itertools.product((2, 3, 4), (2, X)):
    res = one_step(X, Y, Z, plo, phi, TY, S, seg_x, min_ncomp(Z), None, lean=True,
                   esz=esz, **LEAN_PROTOCOL)
    if res is None:
      continue
    reads, bad, cover = res
    assert not bad, (X, Y, Z, TY, plo, phi, S, seg_x, bad[:3])
    assert (cover == 1).all(), (S, seg_x)
    checked += reads
  assert checked > 0


@pytest.mark.parametrize("esz", [4, 2])
def test_lean_items_cover_each_quad_once(esz):
  """Every (row, quad) of the H phase is held exactly once, z-PML quads
  are exactly the slab quads, and a z-PML quad's state column is its
  z-PML column; without the split mapping z-PML quads fill whole warps."""
  for Z, TY, plo, phi in [(64, 14, 8, 8), (48, 19, 4, 12), (32, 29, 0, 0),
                          (64, 14, 12, 0), (64, 14, 0, 0), (64, 28, 16, 16),
                          (64, 14, 4, 24), (64, 14, 12, 24)]:
    thr, rH, z0, col, pml, n = lean_items(Z, TY, plo, phi, esz)
    assert n % 32 == 0 and len(np.unique(thr)) == len(thr)
    live = rH < TY + 1
    pairs = set(zip(rH[live].tolist(), z0[live].tolist()))
    assert len(pairs) == live.sum() == (TY + 1) * Z // 4
    assert (pml[live] == ((z0[live] < plo) | (z0[live] >= Z - phi))).all()
    zp = z0[live & pml]
    zc = np.where(zp < plo, zp, zp - (Z - phi) + plo)
    assert (zc == col[live & pml]).all()
    if not lean_split(Z, plo, phi, esz) and not lean_rows(Z, esz):
      assert len(np.unique(pml.reshape(-1, 32), axis=1)[0]) <= 2


@pytest.mark.parametrize("plo,phi", [(8, 8), (0, 0), (4, 12), (12, 20), (16, 16)])
def test_row_items_are_free_of_bank_conflicts_in_binary16(plo, phi):
  """Binary16 zz 64: every group of 16 lanes (one 128-byte pass of a 64-bit
  shared access) holds 16 distinct bank pairs (quad % 16; rows are 128
  bytes)."""
  for TY in (14, 13, 28):
    thr, rH, z0, _, _, _ = lean_items(64, TY, plo, phi, 2)
    g = ((z0 // 4) % 16).reshape(-1, 16)
    assert all(len(set(row)) == 16 for row in g.tolist())


@pytest.mark.parametrize("Z,esz", [(32, 4), (32, 2), (48, 2), (64, 2)])
@pytest.mark.parametrize("plo,phi", [(8, 8), (0, 0), (4, 12), (16, 16)])
def test_row_major_items_are_free_of_bank_conflicts(Z, esz, plo, phi):
  """Row-major items (zz 32, binary16): lanes hold consecutive quads, so
  each pass (8 lanes of 16 bytes for FP32, 16 lanes of 8 bytes for
  binary16) covers 128 contiguous bytes of a region: distinct banks."""
  quad = 4 * esz              # bytes per quad access
  lanes = 128 // quad          # lanes per 128-byte pass
  for TY in (29, 28, 19, 5):
    thr, rH, z0, _, _, _ = lean_items(Z, TY, plo, phi, esz)
    off = (rH * Z + z0) * esz  # byte offset of the quad in a row-major region
    group = (off // quad) % lanes  # the quad's group of banks
    assert all(len(set(row)) == lanes for row in group.reshape(-1, lanes).tolist())


@pytest.mark.parametrize("plo,phi", [(8, 8), (0, 0), (4, 12), (12, 20), (16, 16)])
def test_split_items_are_free_of_bank_conflicts(plo, phi):
  """FP32 zz 64: in every group of 8 lanes (one 128-byte pass of a 128-bit
  shared access) the quads fall in 8 distinct bank groups (quad % 8; rows
  are 256 bytes), so no quad access of the lean kernels conflicts."""
  for TY in (14, 13, 12):
    thr, rH, z0, _, _, _ = lean_items(64, TY, plo, phi, 4)
    g = ((z0 // 4) % 8).reshape(-1, 8)
    assert all(len(set(row)) == 8 for row in g.tolist())


def test_lean_model_flags_a_planted_mistake():
  """A lean replay whose absorber offset is dropped reads stale data; one
  barrier per plane with only two new-H buffers races."""
  args = (5, 30, 64, 8, 8, 14, 3, 2, 32, None)
  assert one_step(*args, lean=True, **LEAN_PROTOCOL)[1] == []
  two = one_step(*args, lean=True, hbuf=2, barriers=1)
  assert any(b[3] == "race" for b in two[1])  # H(x + 1) over H(x - 1)
  res = one_step(*args, plant="moff", lean=True, **LEAN_PROTOCOL)
  assert any(b[2] == "LE:mask" and b[3] == "stale" for b in res[1])


def lean_geom(TY, Z, P, esz):
  """Byte layout of a lean CTA (``LeanGeom`` in csrc/lean_kernel.cuh): slot
  regions E, H, coefficients (stored type), absorber (FP32), PML state
  (stored type, rows of Pp values); then new H (three buffers), new E, new
  PML state."""
  per16 = 16 // esz
  Pp = (P + per16 - 1) // per16 * per16
  RE, RH, MT = TY + 2, TY + 1, r4(TY) + 8
  e = 0
  h = e + 3 * RE * Z * esz
  c = h + 3 * RH * Z * esz
  m = c + 3 * TY * Z * esz
  p = m + 3 * MT * 4
  stage = p + 4 * RH * Pp * esz
  return dict(Pp=Pp, e=e, h=h, c=c, m=m, p=p, stage=stage,
              hn=3 * 3 * RH * Z * esz, en=2 * 3 * TY * Z * esz,
              pn=2 * 4 * TY * Pp * esz)


@pytest.mark.parametrize("esz", [4, 2])
@pytest.mark.parametrize("Z,TY", [(64, 14), (48, 19), (32, 29), (32, 28)])
@pytest.mark.parametrize("P", [0, 8, 12, 16, 24])
def test_lean_geometry_bulk_copy_alignment(esz, Z, TY, P):
  """Every region a bulk copy fills or drains starts on a 16-byte boundary
  and every copied row (E/H/coefficient rows of Z values, PML state rows of
  Pp values, whole absorber windows) is a whole number of 16-byte units,
  for FP32 and binary16 storage; FP32 is the streamed kernel's layout."""
  g = lean_geom(TY, Z, P, esz)
  for k in ("e", "h", "c", "m", "p", "stage", "hn", "en", "pn"):
    assert g[k] % 16 == 0, (k, g[k])
  assert (Z * esz) % 16 == 0 and (g["Pp"] * esz) % 16 == 0
  assert g["Pp"] >= P and g["Pp"] - P < 16 // esz
  if esz == 4:
    RE, RH, MT = TY + 2, TY + 1, r4(TY) + 8
    stage = 3 * RE * Z + 3 * RH * Z + 3 * TY * Z + 3 * MT + 4 * RH * r4(P)
    assert g["stage"] == 4 * stage
  # Quads (4 values) of every region are 16-byte (FP32) / 8-byte (binary16)
  # aligned: region starts are 16-byte aligned and rows hold whole quads.
  assert Z % 4 == 0 and g["Pp"] % 4 == 0


@pytest.mark.parametrize("esz", [4, 2])
@pytest.mark.parametrize("X,Y,Z,TY", [(6, 40, 64, 14), (5, 23, 64, 14),
                                      (7, 31, 32, 8), (4, 11, 16, 5)])
@pytest.mark.parametrize("plo,phi", [(0, 0), (8, 8), (4, 12)])
def test_lean_two_step_compute_accesses(X, Y, Z, TY, plo, phi, esz):
  """The lean two-step kernel (one quad item per thread over the NR = TY+3
  rows of level 1, interior and PML warps) under the two-step kernel's ring
  protocol: every shared access in bounds and quad-aligned, every read the
  exact data (field, level, plane, row) its update needs, no race between
  barriers, every level-1 and level-2 row of the launch stored once."""
  if plo + phi > Z:
    pytest.skip("slabs wider than the domain")
  checked = 0
  for SA, seg_x in itertools.product((2, 3), (1, 3, X)):
    res = two_step(X, Y, Z, plo, phi, TY, SA, seg_x, min_ncomp(Z), lean=True,
                   esz=esz)
    if res is None:
      continue
    reads, bad, cover = res
    assert not bad, (X, Y, Z, TY, plo, phi, SA, seg_x, bad[:3])
    assert (cover == 1).all(), (SA, seg_x)
    checked += reads
  assert checked > 0
