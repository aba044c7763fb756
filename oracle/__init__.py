"""CPU oracle for the pjz FDTD hot path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker.  The product package
``pjz_gb300`` never imports, links or runs anything here.

Contents:
  * ``yee.c`` -- C restatement of the Yee/CPML update (FP32 with explicit
    fmaf, bit-for-bit the same IEEE operations as the CUDA kernels, and an
    FP64 build), OpenMP over x.  Built by :func:`build` into ``liboracle.so``.
  * ``yee_numpy.py`` -- an independent vectorised NumPy FP64 transcription,
    used to cross-check ``yee.c``.
  * ``pjz_ref.py`` -- NumPy restatement of pjz's ``field`` pre/post-processing
    (``src/pjz/_field.py``), pinned by the golden vectors of the reference's
    own tests.

Parity status: the helpers of ``src/pjz/_field.py`` are pinned by the
reference's test vectors; the engine arithmetic (fdtdz, an absent third-party
CUDA package) is "parity unpinned" -- it is restated from the Yee/CPML
algorithm under pjz's conventions.
"""

import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
  """Compiles ``yee.c`` twice (FP32, FP64) into ``liboracle.so`` with gcc."""
  src = os.path.join(HERE, "yee.c")
  if (not force and os.path.exists(LIB_PATH)
      and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
    return LIB_PATH
  objs = []
  flags = ["-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c11"]
  tag = f"{platform.machine()}_{os.getpid()}"
  for real, name in (("", "f32"), ("-DREAL=double", "f64")):
    obj = os.path.join(HERE, f"yee_{name}_{tag}.o")
    cmd = ["gcc", *flags, "-c", src, "-o", obj] + ([real] if real else [])
    subprocess.run(cmd, check=True)
    objs.append(obj)
  tmp = LIB_PATH + f".{tag}.tmp"
  subprocess.run(["gcc", "-shared", "-fopenmp", *objs, "-o", tmp, "-lm"],
                 check=True)
  os.replace(tmp, LIB_PATH)
  for o in objs:
    os.remove(o)
  return LIB_PATH


class Problem(ctypes.Structure):
  """Mirror of ``oracle_problem`` in ``yee.c``."""
  _fields_ = [(n, ctypes.c_int32) for n in (
      "xx", "yy", "zz", "ox", "oy", "oz", "rx", "ry", "rz", "tt",
      "pml_lo", "pml_hi")] + [("dt", ctypes.c_float)] + [
      (n, ctypes.c_int32) for n in (
          "sx0", "sy0", "sz0", "snx", "sny", "snz", "snc",
          "out_start", "out_stop", "out_step", "mode", "nrows", "record_h",
          "gx0", "gy0", "gz0", "gnx", "gny", "gnz", "nthreads", "storage")]


_lib = None


def _load():
  global _lib
  if _lib is None:
    build()
    _lib = ctypes.CDLL(LIB_PATH)
    for name in ("oracle_run_f32", "oracle_run_f64"):
      fn = getattr(_lib, name)
      fn.restype = ctypes.c_int
      fn.argtypes = [ctypes.POINTER(Problem)] + [ctypes.c_void_p] * 12
    _lib.oracle_round_f16.restype = ctypes.c_float
    _lib.oracle_round_f16.argtypes = [ctypes.c_float]
  return _lib


MODES = {"none": 0, "snapshot": 1, "project": 2, "grad": 3}


def plane_source_box(source_field, source_position, domain):
  """fdtdz plane source -> (box origin, box shape, profile[col][3][box]).

  x/y-normal ``(2, 1, Y, Z)`` / ``(2, X, 1, Z)``: waveform column 0 drives
  plane ``source_position``, column 1 plane ``source_position - 1``; the two
  leading entries are the two transverse E components in xyz order.
  z-normal ``(2, 2, X, Y, 1)``: column k carries profile ``source_field[k]``
  (Ex, Ey) at plane ``source_position``.
  """
  X, Y, Z = domain
  sf = np.asarray(source_field, np.float32)
  s = int(source_position)
  if sf.ndim == 5:
    assert sf.shape == (2, 2, X, Y, 1), sf.shape
    prof = np.zeros((2, 3, X, Y, 1), np.float32)
    prof[:, 0:2] = sf
    return (0, 0, s), (X, Y, 1), prof
  assert sf.ndim == 4 and sf.shape[0] == 2
  axis = 0 if sf.shape[1] == 1 else 1
  assert sf.shape[axis + 1] == 1
  comps = [c for c in range(3) if c != axis]
  lo = max(s - 1, 0)
  n = s + 1 - lo
  shape = [X, Y, Z]
  shape[axis] = n
  prof = np.zeros((2, 3) + tuple(shape), np.float32)
  for col, plane in ((0, s), (1, s - 1)):
    if plane < 0:
      continue
    sl = [slice(None)] * 3
    sl[axis] = slice(plane - lo, plane - lo + 1)
    for k, c in enumerate(comps):
      prof[(col, c) + tuple(sl)] = sf[k]
  origin = [0, 0, 0]
  origin[axis] = lo
  return tuple(origin), tuple(shape), prof


def run(*, eps, offset, mask, kappa, sigma, alpha, dt, tt, pml_widths,
        source_origin, source_profile, waveform, output_steps=(0, 0, 1),
        mode="snapshot", weights=None, q=None, grad_origin=(0, 0, 0),
        record_h=False, fields=None, precision="f32", nthreads=0,
        storage="f32"):
  """Runs ``tt`` Yee steps on the CPU; returns a dict of outputs.

  ``eps`` (3,rx,ry,rz) at ``offset``; ``mask`` (3,X,Y) defines X, Y;
  ``kappa/sigma/alpha`` (Z,2) define Z.  ``source_profile`` is
  ``(ncols, 3, sx, sy, sz)`` at ``source_origin`` with ``waveform (tt,
  ncols)``.  Modes: ``snapshot`` returns E (and H) at ``range(*output_steps)``
  as ``(ns, 3, rx, ry, rz)``; ``project`` returns ``weights @ snapshots``
  (rows x 3 x region) with compensated FP summation; ``grad`` returns the
  per-cell sum over samples of ``E * (weights[:, j] . q)`` over the box
  ``q.shape[2:]`` at ``grad_origin``.  ``storage="f16"`` (with
  ``precision="f32"``) rounds every stored field, CPML state and E-update
  coefficient to binary16, the engine's reduced-precision storage.
  """
  lib = _load()
  real = np.float32 if precision == "f32" else np.float64
  fn = lib.oracle_run_f32 if precision == "f32" else lib.oracle_run_f64
  f32 = lambda a: np.ascontiguousarray(a, np.float32)
  eps, mask = f32(eps), f32(mask)
  kappa, sigma, alpha = f32(kappa), f32(sigma), f32(alpha)
  prof, wave = f32(source_profile), f32(waveform)
  _, X, Y = mask.shape
  Z = kappa.shape[0]
  assert wave.shape == (tt, prof.shape[0]), (wave.shape, tt, prof.shape)
  p = Problem()
  p.xx, p.yy, p.zz = X, Y, Z
  p.ox, p.oy, p.oz = offset
  p.rx, p.ry, p.rz = eps.shape[1:]
  p.tt = tt
  p.pml_lo, p.pml_hi = pml_widths
  p.dt = dt
  p.sx0, p.sy0, p.sz0 = source_origin
  p.snc = prof.shape[0]
  p.snx, p.sny, p.snz = prof.shape[2:]
  p.out_start, p.out_stop, p.out_step = output_steps
  p.mode = MODES[mode]
  p.record_h = int(record_h)
  p.nthreads = nthreads
  if storage not in ("f32", "f16") or (storage == "f16" and precision != "f32"):
    raise ValueError("storage must be 'f32', or 'f16' with precision 'f32'")
  p.storage = 1 if storage == "f16" else 0
  ns = len(range(*output_steps))
  R = (p.rx, p.ry, p.rz)
  out = out_h = None
  wts = qq = None
  if mode == "snapshot":
    out = np.zeros((ns, 3) + R, real)
    out_h = np.zeros((ns, 3) + R, real) if record_h else None
  elif mode == "project":
    wts = f32(weights)
    p.nrows = wts.shape[0]
    assert wts.shape[1] == ns
    out = np.zeros((p.nrows, 3) + R, real)
    out_h = np.zeros((p.nrows, 3) + R, real) if record_h else None
  elif mode == "grad":
    wts, qq = f32(weights), f32(q)
    p.nrows = wts.shape[0]
    assert qq.shape[:2] == (p.nrows, 3)
    p.gx0, p.gy0, p.gz0 = grad_origin
    p.gnx, p.gny, p.gnz = qq.shape[2:]
    out = np.zeros((3,) + qq.shape[2:], real)
  if fields is not None:
    fields = np.ascontiguousarray(fields, real)
    assert fields.shape == (6, X, Y, Z)
  ptr = lambda a: None if a is None else a.ctypes.data
  rc = fn(ctypes.byref(p), ptr(eps), ptr(mask), ptr(kappa), ptr(sigma),
          ptr(alpha), ptr(prof), ptr(wave), ptr(wts), ptr(qq), ptr(fields),
          ptr(out), ptr(out_h))
  if rc != 0:
    raise ValueError(f"oracle rejected the problem (code {rc})")
  return {"out": out, "out_h": out_h, "fields": fields}


def round_f16(v: float) -> float:
  """The oracle's binary16 rounding of one float (round to nearest even)."""
  return float(_load().oracle_round_f16(float(v)))
