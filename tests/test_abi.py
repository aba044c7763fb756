"""C-ABI checks that need no GPU: the library loads, exports every symbol the
header declares, and its host-only plan validation behaves like pjz's
argument checks (bad shapes -> ValueError)."""

import ctypes
import os
import re

import numpy as np
import pytest

from pjz_gb300 import _build, _lib, engine

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include",
                      "pjzfdtd.h")


@pytest.fixture(scope="module")
def lib():
  _build.build()
  return _lib.load()


def declared_symbols():
  text = open(HEADER).read()
  return sorted(set(re.findall(r"\b(pjzfdtd_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
  syms = declared_symbols()
  assert "pjzfdtd_forward" in syms and "pjzfdtd_adjoint" in syms
  assert len(syms) >= 10


def test_library_exports_every_declared_symbol(lib):
  for name in declared_symbols():
    assert hasattr(lib, name), name
  assert set(declared_symbols()) <= set(_lib.SIGNATURES) | set(
      n for n in declared_symbols() if hasattr(lib, n))


def test_abi_version(lib):
  assert lib.pjzfdtd_abi_version() == 2


def test_struct_sizes_match_header():
  # 12 ints + float + 28 ints = 41 x 4 bytes.
  assert ctypes.sizeof(_lib.Problem) == 164
  assert ctypes.sizeof(_lib.Buffers) == 8 * 8


def _plan(**kw):
  Z = kw.pop("Z", 16)
  base = dict(domain=(20, 18, Z), offset=(2, 2, 2), region=(16, 14, Z - 4),
              tt=50, dt=0.5, pml_widths=(2, 2),
              pml_kappa=np.ones((Z, 2)), pml_sigma=np.zeros((Z, 2)),
              pml_alpha=np.zeros((Z, 2)), source_origin=(4, 0, 0),
              source_shape=(2, 18, Z), source_ncols=2,
              output_steps=(30, 50, 5), out_mode=engine.OUT_SNAPSHOTS)
  base.update(kw)
  return engine.Plan(**base)


def test_plan_create_host_only(lib):
  p = _plan()
  assert p.num_samples == 4
  X, Y, Z = p.domain
  assert p.workspace_bytes >= (15 * X * Y * Z) * 4
  cfg = p.launch_config()
  assert cfg["kernel"] == 2 and cfg["stages"] >= 2  # zz % 4 == 0: streamed
  assert 1 <= cfg["tile_y"] <= Y and cfg["threads"] % 32 == 0
  q = _plan(kernel=1)
  cfg = q.launch_config()
  assert cfg["kernel"] == 1 and cfg["threads"] % 32 == 0
  assert (cfg["tile_y"] + 2) * Z <= cfg["threads"]
  r = _plan(Z=18, region=(16, 14, 14), source_shape=(2, 18, 18))
  assert r.launch_config()["kernel"] == 1  # zz % 4 != 0 falls back


@pytest.mark.parametrize("bad,msg", [
    (dict(offset=(5, 2, 2)), "does not fit"),
    (dict(pml_widths=(10, 10)), "pml_widths"),
    (dict(dt=-1.0), "dt must be positive"),
    (dict(source_origin=(19, 0, 0)), "source box"),
    (dict(output_steps=(30, 60, 5)), "output_steps"),
    (dict(output_steps=(30, 30, 5)), "output_steps"),
    (dict(output_steps=(30, 50, 0)), "output step"),
    (dict(pml_kappa=np.zeros((16, 2))), "kappa > 0"),
    (dict(pml_sigma=-np.ones((16, 2))), "sigma >= 0"),
    (dict(pml_kappa=np.ones((15, 2))), "must have shape"),
    (dict(out_mode=engine.OUT_PHASORS, weights=np.ones((40, 4))), "out_rows"),
])
def test_plan_create_rejects(lib, bad, msg):
  with pytest.raises(ValueError, match=msg):
    _plan(**bad)


def test_thick_z_is_unsupported_not_silent(lib):
  with pytest.raises(NotImplementedError, match="thin-z"):
    _plan(Z=401, region=(16, 14, 300), offset=(2, 2, 2),
          source_shape=(2, 18, 401))
  with pytest.raises(ValueError, match="zz % 4"):
    _plan(kernel=2, Z=18, region=(16, 14, 14), source_shape=(2, 18, 18))


def test_kappa_inf_allowed(lib):
  # use_z_as_batch (pjz _field.py:243-246) passes kappa = inf.
  _plan(pml_kappa=np.full((16, 2), np.inf))


def test_last_error_is_thread_local_message(lib):
  with pytest.raises(ValueError):
    _plan(dt=0.0)
  assert "dt" in _lib.last_error()


def test_negative_output_start_is_allowed(lib):
  # pjz asks for samples before step 0 when tt < 2 * interval * ww + 1.
  p = _plan(output_steps=(-12, 50, 9))
  assert p.num_samples == len(range(-12, 50, 9))


@pytest.mark.parametrize("Z", [64, 48, 32])
@pytest.mark.parametrize("pml", [(8, 8), (4, 4), (0, 0), (4, 8), (12, 4)])
def test_lean_kernel_plans_resolve(lib, Z, pml):
  """kernel=3 (lean) resolves on every thin-z shape it is tested with on the
  GPU: a compile-time tile, one step per launch, interior plus PML warps
  within the block bound; uneven slab widths are refused."""
  import sys
  sys.path.insert(0, os.path.dirname(__file__))
  from _cases import random_problem
  case = random_problem(1, X=19, Y=2 * {64: 14, 48: 19, 32: 29}[Z] + 5, Z=Z,
                        pml=pml, tt=24, steps=(9, 24, 4))
  kw = dict(domain=case["domain"], offset=case["offset"],
            region=case["eps"].shape[1:], tt=24, dt=0.5, pml_widths=pml,
            pml_kappa=case["kappa"], pml_sigma=case["sigma"],
            pml_alpha=case["alpha"], source_origin=case["source_origin"],
            source_shape=case["source_profile"].shape[2:], source_ncols=2,
            output_steps=(9, 24, 4), out_mode=engine.OUT_SNAPSHOTS, kernel=3)
  cfg = engine.Plan(**kw).launch_config()
  assert cfg["kernel"] == 3 and cfg["steps_per_pass"] == 1
  assert (Z, cfg["tile_y"]) in {(64, 14), (48, 19), (32, 29), (32, 28)}
  assert cfg["threads"] <= 384 and cfg["threads"] % 32 == 0
  with pytest.raises(NotImplementedError, match="lean"):
    engine.Plan(**dict(kw, pml_widths=(3, 5), pml_kappa=np.ones((Z, 2)),
                       pml_sigma=np.zeros((Z, 2)), pml_alpha=np.zeros((Z, 2))))


@pytest.mark.parametrize("Z,pml,ok", [(64, (8, 8), True), (48, (4, 4), True),
                                      (32, (8, 8), True), (64, (3, 5), False),
                                      (40, (8, 8), False), (18, (3, 2), False)])
def test_binary16_storage_plans(lib, Z, pml, ok):
  """storage=1 (binary16) resolves to the lean kernel where it applies and
  is refused elsewhere; its workspace holds 2-byte fields, coefficients and
  z-PML state (state rows padded to 8 values)."""
  Y = 33 if Z != 32 else 61
  kw = dict(domain=(20, Y, Z), offset=(2, 2, 2), region=(16, Y - 4, Z - 4),
            tt=50, dt=0.5, pml_widths=pml, pml_kappa=np.ones((Z, 2)),
            pml_sigma=np.zeros((Z, 2)), pml_alpha=np.zeros((Z, 2)),
            source_origin=(4, 0, 0), source_shape=(2, Y, Z), source_ncols=2,
            output_steps=(30, 50, 5), out_mode=engine.OUT_SNAPSHOTS)
  if not ok:
    with pytest.raises(NotImplementedError):
      engine.Plan(**kw, storage=engine.STORAGE_F16)
    return
  half = engine.Plan(**kw, storage=engine.STORAGE_F16)
  full = engine.Plan(**kw)
  assert half.launch_config()["kernel"] == 3
  N = 20 * Y * Z
  # 15 N stored values (two states of 6, 3 coefficients) per plan.
  assert full.workspace_bytes - half.workspace_bytes >= 15 * N * 2 - 4096
  with pytest.raises(NotImplementedError, match="lean"):
    engine.Plan(**kw, storage=engine.STORAGE_F16, kernel=2)
  with pytest.raises(ValueError, match="storage"):
    engine.Plan(**kw, storage=2)


def test_binary16_plans_stay_out_of_batches(lib):
  Z = 64
  kw = dict(domain=(20, 33, Z), offset=(0, 0, 0), region=(20, 33, Z), tt=20,
            dt=0.5, pml_widths=(8, 8), pml_kappa=np.ones((Z, 2)),
            pml_sigma=np.zeros((Z, 2)), pml_alpha=np.zeros((Z, 2)))
  with pytest.raises(NotImplementedError, match="binary16"):
    engine.Batch([engine.Plan(**kw, storage=engine.STORAGE_F16)])


@pytest.mark.parametrize("pml,ok", [((0, 0), True), ((8, 8), True), ((4, 12), True),
                                    ((12, 12), True), ((6, 6), False)])
def test_tall_binary16_tile(lib, pml, ok):
  """tile_y=28 at zz 64 with binary16 storage takes the tall lean tile (two
  rows per warp, 15 compute warps for any slab widths); slabs that are not
  whole quads are refused.  FP32 has no such tile."""
  Z = 64
  kw = dict(domain=(20, 61, Z), offset=(0, 0, 0), region=(20, 61, Z), tt=20,
            dt=0.5, pml_widths=pml, pml_kappa=np.ones((Z, 2)),
            pml_sigma=np.zeros((Z, 2)), pml_alpha=np.zeros((Z, 2)), tile_y=28)
  if not ok:
    with pytest.raises(NotImplementedError, match="multiples of 4"):
      engine.Plan(**kw, storage=engine.STORAGE_F16)
    return
  cfg = engine.Plan(**kw, storage=engine.STORAGE_F16).launch_config()
  assert cfg["kernel"] == 3 and cfg["tile_y"] == 28
  assert cfg["threads"] <= 512 and cfg["threads"] % 32 == 0
  with pytest.raises(ValueError, match="exceeds shared"):
    engine.Plan(**kw)


def test_auto_takes_the_lean_kernels_and_batches_fall_back(lib):
  """FP32 plans with kernel and steps per pass automatic run the lean
  two-step kernel where its compile-time shape applies (zz 64, tile_y 14),
  else the lean one-step kernel; a batch takes such a plan on the streamed
  plan it replaced (same workspace), while a plan that asked for the lean
  kernel stays out of batches."""
  Z = 64
  kw = dict(domain=(40, 56, Z), offset=(0, 0, 0), region=(40, 56, Z), tt=20,
            dt=0.5, pml_widths=(8, 8), pml_kappa=np.ones((Z, 2)),
            pml_sigma=np.zeros((Z, 2)), pml_alpha=np.zeros((Z, 2)),
            source_origin=(6, 0, 0), source_shape=(2, 56, Z), source_ncols=2)
  auto = engine.Plan(**kw)
  cfg = auto.launch_config()
  assert (cfg["kernel"], cfg["steps_per_pass"], cfg["tile_y"]) == (3, 2, 14)
  one = engine.Plan(**kw, steps_per_pass=1).launch_config()
  assert (one["kernel"], one["steps_per_pass"]) == (3, 1)
  streamed = engine.Plan(**kw, kernel=2)
  ws = auto.workspace_bytes
  assert ws == streamed.workspace_bytes
  engine.Batch([auto])
  cfg = auto.launch_config()
  assert (cfg["kernel"], cfg["steps_per_pass"]) == (2, 1)
  assert auto.workspace_bytes == ws
  with pytest.raises(NotImplementedError, match="lean kernel by request"):
    engine.Batch([engine.Plan(**kw, kernel=3)])
  # odd z-PML widths or a y-normal box that rides the ring keep the streamed
  # kernels
  odd = dict(kw, pml_widths=(6, 6))
  assert engine.Plan(**odd).launch_config()["kernel"] == 2
