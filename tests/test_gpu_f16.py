"""Reduced-precision storage on the GB300: binary16 fields, coefficients and
z-PML state with FP32 arithmetic (``storage=1``, what pjz's default
``use_reduced_precision=True`` selects, ``src/pjz/_field.py:52``).

The lean kernel rounds every stored value to nearest even exactly where the
FP32 oracle run with ``storage="f16"`` does, so the snapshots, phasors,
recorded H and final state are bit-identical to that oracle.  Against the
FP64 oracle the c0 waveguide (2000 steps) is held to 5e-3 relative L2 (the
FP32 engine: 1e-5); the measured figure is printed."""

import numpy as np
import pytest
import torch

import oracle
import pjz_gb300
from pjz_gb300 import engine, workloads
from _cases import field_oracle, oracle_kwargs, random_problem
from test_gpu_forward import gpu_run

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")
F16 = engine.STORAGE_F16


def gpu16(case, **kw):
  return gpu_run(case, storage=F16, **kw)


@pytest.mark.parametrize("Z,TY", [(64, 14), (48, 19), (32, 28)])
@pytest.mark.parametrize("pml", [(8, 8), (4, 4), (0, 0), (4, 12)])
@pytest.mark.parametrize("src", ["x", "y", "z"])
def test_f16_snapshots_bit_exact(native, Z, TY, pml, src):
  case = random_problem(hash((Z, pml, src, 16)) % 1000, X=19, Y=2 * TY + 5, Z=Z,
                        pml=pml, src=src, src_pos=5 if src == "z" else 7,
                        tt=24, steps=(9, 24, 4))
  want = oracle.run(**oracle_kwargs(case), storage="f16")["out"]
  got, _, _ = gpu16(case, seg_x=6, tile_y=TY)
  assert np.array_equal(got, want), np.abs(got - want).max()


@pytest.mark.parametrize("pml", [(8, 8), (0, 0), (4, 12)])
@pytest.mark.parametrize("src", ["x", "y", "z"])
@pytest.mark.parametrize("stages,seg_x", [(0, 6), (3, 19), (2, 4)])
def test_f16_tall_tile_bit_exact(native, pml, src, stages, seg_x):
  """The tall binary16 tile (zz 64, tile_y 28, up to 16 warps) with a
  ragged last tile, over ring depths and segments."""
  case = random_problem(hash((pml, src, stages, 28)) % 1000, X=19, Y=61, Z=64,
                        pml=pml, src=src, src_pos=5 if src == "z" else 7,
                        tt=24, steps=(9, 24, 4))
  want = oracle.run(**oracle_kwargs(case), storage="f16")["out"]
  got, _, _ = gpu16(case, tile_y=28, stages=stages, seg_x=seg_x)
  assert np.array_equal(got, want), np.abs(got - want).max()


def test_f16_tall_tile_phasors_state_and_chaining(native):
  case = random_problem(52, X=17, Y=70, Z=64, pml=(8, 8), tt=40, steps=(10, 40, 3))
  ns = len(range(*case["output_steps"]))
  w = np.random.default_rng(7).normal(size=(6, ns)).astype(np.float32)
  f0 = np.random.default_rng(8).normal(size=(6,) + case["domain"]).astype(np.float32)
  want = oracle.run(**oracle_kwargs(case), mode="project", weights=w, record_h=True,
                    fields=f0.copy(), storage="f16")
  got, got_h, got_f = gpu16(case, out_mode=engine.OUT_PHASORS, weights=w,
                            record_h=True, fields=f0.copy(), tile_y=28)
  assert np.array_equal(got, want["out"])
  assert np.array_equal(got_h, want["out_h"])
  assert np.array_equal(got_f, want["fields"])
  snap = oracle.run(**oracle_kwargs(case), storage="f16")["out"]
  got, _, _ = gpu16(case, split=17, tile_y=28)
  assert np.array_equal(got, snap)


def test_f16_phasors_record_h_state_and_chaining(native):
  case = random_problem(51, X=17, Y=30, Z=64, pml=(8, 8), tt=40, steps=(10, 40, 3))
  ns = len(range(*case["output_steps"]))
  w = np.random.default_rng(6).normal(size=(6, ns)).astype(np.float32)
  f0 = np.random.default_rng(9).normal(size=(6,) + case["domain"]).astype(np.float32)
  want = oracle.run(**oracle_kwargs(case), mode="project", weights=w, record_h=True,
                    fields=f0.copy(), storage="f16")
  got, got_h, got_f = gpu16(case, out_mode=engine.OUT_PHASORS, weights=w,
                            record_h=True, fields=f0.copy())
  assert np.array_equal(got, want["out"])
  assert np.array_equal(got_h, want["out_h"])
  assert np.array_equal(got_f, want["fields"])
  snap = oracle.run(**oracle_kwargs(case), storage="f16")["out"]
  got, _, _ = gpu16(case, split=17)
  assert np.array_equal(got, snap)


def test_f16_field_c0_vs_oracles(native):
  """``field`` with use_reduced_precision=True on c0 (128x128x32, 2000
  steps): bit-exact to the FP32 oracle with binary16 storage, within 5e-3
  of the FP64 oracle."""
  wl = workloads.waveguide_c0()
  sp = wl.sim_params._replace(use_reduced_precision=True)
  wl16 = wl._replace(sim_params=sp)
  got = pjz_gb300.field(torch.as_tensor(wl.epsilon, device=DEV),
                        torch.as_tensor(wl.source, device=DEV), wl.omega,
                        wl.source_pos, sp).cpu().numpy()
  want16 = field_oracle(wl16, "f32", storage="f16").astype(np.complex64)
  assert np.array_equal(got, want16), np.abs(got - want16).max()
  want64 = field_oracle(wl, "f64")
  err = np.linalg.norm(got - want64) / np.linalg.norm(want64)
  print(f"\nc0 binary16 storage vs FP64 oracle: rel-L2 {err:.3e}")
  assert err < 5e-3


def test_f16_fdtdz_dropin_flag(native):
  """pjz's fdtdz keyword use_reduced_precision=True selects the storage."""
  case = random_problem(52, X=16, Y=33, Z=64, pml=(8, 8), src="y", src_pos=6)
  out = pjz_gb300.fdtdz(
      epsilon=torch.as_tensor(case["eps"], device=DEV), dt=0.5,
      source_field=torch.as_tensor(case["source_field"], device=DEV),
      source_waveform=torch.as_tensor(case["waveform"], device=DEV),
      source_position=6, absorption_mask=torch.as_tensor(case["mask"], device=DEV),
      pml_kappa=case["kappa"], pml_sigma=case["sigma"], pml_alpha=case["alpha"],
      pml_widths=case["pml_widths"], output_steps=case["output_steps"],
      use_reduced_precision=True, launch_params=None, offset=case["offset"])
  want = oracle.run(**oracle_kwargs(case), storage="f16")["out"]
  assert np.array_equal(out.cpu().numpy(), want)
