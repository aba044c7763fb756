"""GPU parity of the lean streamed kernel (``kernel=3``,
``csrc/lean_kernel.cuh``) against the CPU oracle, bit for bit: every
compile-time shape, z-PML slab widths that are multiples of 4 (including
none and uneven slabs), every source orientation, tile and segment
boundaries inside the domain, ring depths, recorded H and final state,
chained partial runs, phasor projection and the 512x512x64 c1 domain."""

import numpy as np
import pytest
import torch

import oracle
from oracle import pjz_ref
from pjz_gb300 import engine, workloads
from _cases import oracle_kwargs, random_problem
from test_gpu_forward import gpu_run

pytestmark = pytest.mark.gpu
SHAPES = [(64, 14), (48, 19), (32, 29)]


@pytest.mark.parametrize("Z,TY", SHAPES)
@pytest.mark.parametrize("pml", [(8, 8), (4, 4), (0, 0), (4, 8), (12, 4)])
@pytest.mark.parametrize("src", ["x", "y", "z"])
def test_lean_snapshots_bit_exact(native, Z, TY, pml, src):
  case = random_problem(hash((Z, pml, src)) % 1000, X=19, Y=2 * TY + 5, Z=Z,
                        pml=pml, src=src, src_pos=5 if src == "z" else 7,
                        tt=24, steps=(9, 24, 4))
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, kernel=3, seg_x=6)
  assert np.array_equal(got, want), np.abs(got - want).max()


@pytest.mark.parametrize("stages,seg_x", [(2, 1), (3, 4), (4, 19), (3, 2)])
def test_lean_ring_and_segments(native, stages, seg_x):
  # The ring depth changes the tile the host picks, so the tile is pinned.
  case = random_problem(31, X=19, Y=33, Z=64, pml=(8, 8), tt=20, steps=(4, 20, 3))
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, kernel=3, tile_y=14, stages=stages, seg_x=seg_x)
  assert np.array_equal(got, want)


def test_lean_record_h_final_state_and_chaining(native):
  case = random_problem(32, X=17, Y=30, Z=64, pml=(8, 8), tt=40, steps=(10, 40, 6))
  f0 = np.random.default_rng(9).normal(size=(6,) + case["domain"]).astype(np.float32)
  want = oracle.run(**oracle_kwargs(case), record_h=True, fields=f0.copy())
  got, got_h, got_f = gpu_run(case, kernel=3, record_h=True, fields=f0.copy())
  assert np.array_equal(got, want["out"])
  assert np.array_equal(got_h, want["out_h"])
  assert np.array_equal(got_f, want["fields"])
  got, _, _ = gpu_run(case, kernel=3, split=23)
  assert np.array_equal(got, oracle.run(**oracle_kwargs(case))["out"])


def test_lean_phasors_bit_exact(native):
  case = random_problem(33, X=18, Y=31, Z=48, pml=(8, 8), tt=48, steps=(10, 48, 3))
  ns = len(range(*case["output_steps"]))
  w = np.random.default_rng(4).normal(size=(10, ns)).astype(np.float32)
  want = oracle.run(**oracle_kwargs(case), mode="project", weights=w)
  got, _, _ = gpu_run(case, out_mode=engine.OUT_PHASORS, weights=w, kernel=3)
  assert np.array_equal(got, want["out"])


def test_lean_refuses_what_it_does_not_cover(native):
  case = random_problem(34, X=12, Y=33, Z=64, pml=(3, 5))
  with pytest.raises(NotImplementedError, match="lean"):
    gpu_run(case, kernel=3)
  case = random_problem(35, X=12, Y=33, Z=40, pml=(8, 8))
  with pytest.raises(NotImplementedError, match="lean"):
    gpu_run(case, kernel=3)


def test_lean_c1_domain_short_run_bit_exact(native):
  """The 512x512x64 c1 domain (x-normal source over two planes, 8-cell
  z-PML) for 24 steps."""
  wl = workloads.design_c1(tt=24, ww=5)
  sp = wl.sim_params
  kw, omega = pjz_ref.field_setup(wl.epsilon, wl.source, wl.omega, wl.source_pos,
                                  pjz_ref.SimParams(*sp[:-1]), zz=wl.domain[2])
  org, shp, prof = oracle.plane_source_box(kw["source_field"],
                                           kw["source_position"], wl.domain)
  case = dict(eps=kw["epsilon"], offset=kw["offset"], mask=kw["absorption_mask"],
              kappa=kw["pml_kappa"], sigma=kw["pml_sigma"], alpha=kw["pml_alpha"],
              dt=0.5, tt=24, pml_widths=kw["pml_widths"], source_origin=org,
              source_profile=prof, waveform=kw["source_waveform"],
              output_steps=(10, 24, 4), domain=wl.domain)
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, kernel=3)
  assert np.array_equal(got, want)


# ---- lean two-step kernel (kernel=3, steps_per_pass=2) ----

STORES = [(engine.STORAGE_F32, "f32"), (engine.STORAGE_F16, "f16")]


@pytest.mark.parametrize("storage,ostore", STORES, ids=["f32", "f16"])
@pytest.mark.parametrize("pml", [(8, 8), (4, 4), (0, 0), (4, 12)])
@pytest.mark.parametrize("src", ["x", "y", "z"])
def test_lean2_snapshots_bit_exact(native, storage, ostore, pml, src):
  """Two steps per launch with the lean compute path, a tile boundary and
  segment boundaries inside the domain: bit-identical to the oracle (FP32,
  or binary16 storage)."""
  case = random_problem(hash((pml, src, 2)) % 1000, X=19, Y=33, Z=64, pml=pml,
                        src=src, src_pos=5 if src == "z" else 7, tt=25,
                        steps=(9, 25, 4))
  want = oracle.run(**oracle_kwargs(case), storage=ostore)["out"]
  got, _, _ = gpu_run(case, kernel=3, steps_per_pass=2, seg_x=6, storage=storage)
  assert np.array_equal(got, want), np.abs(got - want).max()


@pytest.mark.parametrize("storage,ostore", STORES, ids=["f32", "f16"])
@pytest.mark.parametrize("tt,steps", [(47, (5, 47, 3)), (40, (0, 40, 1)),
                                      (41, (-6, 41, 2)), (9, (8, 9, 1))])
def test_lean2_schedule_around_samples(native, storage, ostore, tt, steps):
  """Two steps per launch except where a sampled state sits between them,
  the sampled steps run by the lean one-step kernel: odd and even sample
  steps, every step sampled, odd tt, samples before step 0; with recorded H
  and final state."""
  case = random_problem(61, X=15, Y=30, Z=64, pml=(8, 8), tt=tt, steps=steps)
  f0 = np.random.default_rng(3).normal(size=(6,) + case["domain"]).astype(np.float32)
  want = oracle.run(**oracle_kwargs(case), record_h=True, fields=f0.copy(),
                    storage=ostore)
  got, got_h, got_f = gpu_run(case, kernel=3, steps_per_pass=2, record_h=True,
                              fields=f0.copy(), seg_x=4, storage=storage)
  assert np.array_equal(got, want["out"])
  assert np.array_equal(got_h, want["out_h"])
  assert np.array_equal(got_f, want["fields"])


@pytest.mark.parametrize("storage,ostore", STORES, ids=["f32", "f16"])
def test_lean2_phasors_chaining_and_segments(native, storage, ostore):
  case = random_problem(62, X=21, Y=31, Z=64, pml=(8, 8), tt=48, steps=(10, 48, 3))
  ns = len(range(*case["output_steps"]))
  w = np.random.default_rng(4).normal(size=(10, ns)).astype(np.float32)
  want = oracle.run(**oracle_kwargs(case), mode="project", weights=w,
                    storage=ostore)["out"]
  for seg_x, split in ((1, None), (5, 23), (21, None)):
    got, _, _ = gpu_run(case, out_mode=engine.OUT_PHASORS, weights=w, kernel=3,
                        steps_per_pass=2, seg_x=seg_x, split=split,
                        storage=storage)
    assert np.array_equal(got, want), (seg_x, split)


def test_lean2_c1_domain_short_run_bit_exact(native):
  """The 512x512x64 c1 domain for 25 steps, two per launch."""
  wl = workloads.design_c1(tt=25, ww=5)
  sp = wl.sim_params
  kw, omega = pjz_ref.field_setup(wl.epsilon, wl.source, wl.omega, wl.source_pos,
                                  pjz_ref.SimParams(*sp[:-1]), zz=wl.domain[2])
  org, shp, prof = oracle.plane_source_box(kw["source_field"],
                                           kw["source_position"], wl.domain)
  case = dict(eps=kw["epsilon"], offset=kw["offset"], mask=kw["absorption_mask"],
              kappa=kw["pml_kappa"], sigma=kw["pml_sigma"], alpha=kw["pml_alpha"],
              dt=0.5, tt=25, pml_widths=kw["pml_widths"], source_origin=org,
              source_profile=prof, waveform=kw["source_waveform"],
              output_steps=(10, 25, 4), domain=wl.domain)
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, kernel=3, steps_per_pass=2)
  assert np.array_equal(got, want)
