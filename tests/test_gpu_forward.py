"""GPU parity of the forward engine against the CPU oracle.

The FP32 engine performs the same IEEE operations in the same order as the
FP32 oracle (``oracle/yee.c``), so every comparison here is bit-exact
(``np.array_equal``); the error against the FP64 oracle is stated with a
1e-5 relative-L2 bound.  All calls go through the C ABI.
"""

import numpy as np
import pytest
import torch

import oracle
from oracle import pjz_ref
from pjz_gb300 import engine, workloads
import pjz_gb300
from _cases import field_oracle, oracle_kwargs, random_problem

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def dev(a):
  return torch.as_tensor(np.ascontiguousarray(a), device=DEV)


def gpu_run(case, out_mode=engine.OUT_SNAPSHOTS, weights=None, record_h=False,
            tile_y=0, seg_x=0, fields=None, split=None, kernel=0, stages=0,
            steps_per_pass=0, storage=engine.STORAGE_F32):
  p = engine.Plan(domain=case["domain"], offset=case["offset"],
                  region=case["eps"].shape[1:], tt=case["tt"], dt=case["dt"],
                  pml_widths=case["pml_widths"], pml_kappa=case["kappa"],
                  pml_sigma=case["sigma"], pml_alpha=case["alpha"],
                  source_origin=case["source_origin"],
                  source_shape=case["source_profile"].shape[2:],
                  source_ncols=case["source_profile"].shape[0],
                  output_steps=case["output_steps"], out_mode=out_mode,
                  weights=weights, record_h=record_h, tile_y=tile_y,
                  seg_x=seg_x, kernel=kernel, stages=stages,
                  steps_per_pass=steps_per_pass, storage=storage)
  if steps_per_pass:
    assert p.launch_config()["steps_per_pass"] == steps_per_pass
  args = dict(epsilon=dev(case["eps"]), absorption_mask=dev(case["mask"]),
              source=dev(case["source_profile"]), waveform=dev(case["waveform"]))
  f = None if fields is None else dev(fields)
  if split is None:
    out, out_h = p.run(**args, fields=f)
  else:
    out, out_h = p.run(**args, fields=f, steps=(0, split))
    out, out_h = p.run(**args, fields=f, out=out, out_h=out_h,
                       steps=(split, case["tt"]))
  torch.cuda.synchronize()
  p.check_status()
  cpu = lambda t: None if t is None else t.cpu().numpy()
  return cpu(out), cpu(out_h), cpu(f)


# register-marching; bulk-copy streamed one step per launch; streamed two
# steps per launch (temporal blocking)
VARIANTS = [dict(kernel=1), dict(kernel=2, steps_per_pass=1),
            dict(kernel=2, steps_per_pass=2)]
VIDS = ["reg", "stream1", "stream2"]


@pytest.mark.parametrize("variant", VARIANTS, ids=VIDS)
@pytest.mark.parametrize("src", ["x", "y", "z"])
@pytest.mark.parametrize("Z,pml", [(16, (2, 2)), (24, (3, 5)), (48, (8, 8)),
                                   (64, (8, 8)), (12, (0, 0))])
def test_snapshots_bit_exact(native, src, Z, pml, variant):
  case = random_problem(hash((src, Z)) % 1000, Z=Z, pml=pml, src=src,
                        src_pos=5 if src == "z" else 7)
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, **variant)
  assert np.array_equal(got, want), np.abs(got - want).max()


def test_odd_z_uses_register_marching_kernel(native):
  case = random_problem(11, Z=18, pml=(3, 2))
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case)
  assert np.array_equal(got, want)


@pytest.mark.parametrize("variant", VARIANTS, ids=VIDS)
def test_use_z_as_batch_bit_exact(native, variant):
  case = random_problem(3, Z=20, batch=True, pml=(0, 0))
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, **variant)
  assert np.array_equal(got, want)


@pytest.mark.parametrize("variant", VARIANTS, ids=VIDS)
@pytest.mark.parametrize("tile_y,seg_x", [(1, 1), (2, 3), (5, 24), (7, 8), (0, 2)])
def test_launch_geometry_does_not_change_results(native, tile_y, seg_x, variant):
  case = random_problem(4, X=26, Y=23, Z=16)
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, tile_y=tile_y, seg_x=seg_x, **variant)
  assert np.array_equal(got, want)


@pytest.mark.parametrize("spp", [1, 2])
@pytest.mark.parametrize("stages", [2, 3, 5, 8])
def test_stream_ring_depth_does_not_change_results(native, stages, spp):
  case = random_problem(12, X=30, Y=21, Z=32, pml=(4, 4))
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, kernel=2, stages=stages, tile_y=6, seg_x=7,
                      steps_per_pass=spp)
  assert np.array_equal(got, want)


@pytest.mark.parametrize("tt,steps", [(47, (5, 47, 3)), (40, (0, 40, 1)),
                                      (41, (-6, 41, 2)), (9, (8, 9, 1))])
def test_two_step_schedule_around_samples(native, tt, steps):
  """Two steps per launch except where a sampled state sits between them:
  odd and even sample steps, every step sampled, odd tt, and sample steps
  before 0.  Results stay bit-identical to the oracle."""
  case = random_problem(13, X=22, Y=19, Z=16, pml=(2, 3), tt=tt, steps=steps)
  want = oracle.run(**oracle_kwargs(case), record_h=True)
  got, got_h, _ = gpu_run(case, kernel=2, steps_per_pass=2, record_h=True,
                          tile_y=4, seg_x=5)
  assert np.array_equal(got, want["out"])
  assert np.array_equal(got_h, want["out_h"])


@pytest.mark.parametrize("Z,tile_y", [(64, 14), (64, 11), (64, 10), (48, 15)])
@pytest.mark.parametrize("pml", [(8, 8), (3, 5), (0, 0)])
@pytest.mark.parametrize("src", ["x", "z"])
def test_two_step_specialised_shapes(native, Z, tile_y, pml, src):
  """The compile-time (zz, tile_y) shapes of the two-step kernel (z-pairs
  straddling a slab edge when a PML width is odd) are bit-identical to the
  oracle, with a tile boundary inside the domain."""
  case = random_problem(15, X=19, Y=2 * tile_y + 5, Z=Z, pml=pml, src=src,
                        tt=24, steps=(9, 24, 4))
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, kernel=2, steps_per_pass=2, tile_y=tile_y, seg_x=6)
  assert np.array_equal(got, want)


@pytest.mark.parametrize("Z,tile_y,stages", [(64, 14, 4), (48, 19, 4), (32, 29, 3)])
@pytest.mark.parametrize("pml", [(8, 8), (3, 5)])
@pytest.mark.parametrize("src", ["x", "y", "z"])
def test_one_step_specialised_shapes(native, Z, tile_y, stages, pml, src):
  """The compile-time (zz, tile_y) shapes of the one-step streamed kernel
  with every source orientation (so both the global-load and ring-carried
  source paths) are bit-identical to the oracle, with a tile boundary
  inside the domain."""
  case = random_problem(16, X=19, Y=2 * tile_y + 5, Z=Z, pml=pml, src=src,
                        src_pos=5 if src == "z" else 7, tt=24, steps=(9, 24, 4))
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, kernel=2, steps_per_pass=1, tile_y=tile_y,
                      stages=stages, seg_x=6)
  assert np.array_equal(got, want)


def test_two_step_rejected_for_register_kernel(native):
  case = random_problem(14, Z=18, pml=(3, 2))
  with pytest.raises(NotImplementedError, match="two steps"):
    gpu_run(case, kernel=1, steps_per_pass=2)


@pytest.mark.parametrize("variant", VARIANTS, ids=VIDS)
def test_record_h_and_final_state(native, variant):
  case = random_problem(5, Z=24, pml=(4, 4))
  f0 = np.random.default_rng(9).normal(size=(6,) + case["domain"]).astype(np.float32)
  want = oracle.run(**oracle_kwargs(case), record_h=True, fields=f0.copy())
  got, got_h, got_f = gpu_run(case, record_h=True, fields=f0.copy(),
                              **variant)
  assert np.array_equal(got, want["out"])
  assert np.array_equal(got_h, want["out_h"])
  assert np.array_equal(got_f, want["fields"])


@pytest.mark.parametrize("variant", VARIANTS, ids=VIDS)
def test_run_steps_chaining_matches_single_run(native, variant):
  case = random_problem(6, tt=60, steps=(20, 60, 7))
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, split=33, **variant)
  assert np.array_equal(got, want)


@pytest.mark.parametrize("variant", VARIANTS, ids=VIDS)
@pytest.mark.parametrize("rows", [2, 10, 32])
def test_phasor_projection_bit_exact(native, rows, variant):
  case = random_problem(7, Z=32, pml=(4, 4), steps=(10, 48, 3))
  ns = len(range(*case["output_steps"]))
  w = np.random.default_rng(rows).normal(size=(rows, ns)).astype(np.float32)
  want = oracle.run(**oracle_kwargs(case), mode="project", weights=w,
                    record_h=True)
  got, got_h, _ = gpu_run(case, out_mode=engine.OUT_PHASORS, weights=w,
                          record_h=True, **variant)
  assert np.array_equal(got, want["out"])
  assert np.array_equal(got_h, want["out_h"])


def test_fdtdz_dropin_matches_oracle(native):
  case = random_problem(8, src="y", src_pos=6, Z=16)
  out = pjz_gb300.fdtdz(
      epsilon=dev(case["eps"]), dt=0.5, source_field=dev(case["source_field"]),
      source_waveform=dev(case["waveform"]), source_position=6,
      absorption_mask=dev(case["mask"]), pml_kappa=case["kappa"],
      pml_sigma=case["sigma"], pml_alpha=case["alpha"],
      pml_widths=case["pml_widths"], output_steps=case["output_steps"],
      use_reduced_precision=False, launch_params=None, offset=case["offset"])
  want = oracle.run(**oracle_kwargs(case))["out"]
  assert np.array_equal(out.cpu().numpy(), want)


_field_oracle = field_oracle


def test_field_short_c0_bit_exact(native):
  wl = workloads.waveguide_c0(tt=400)
  got = pjz_gb300.field(dev(wl.epsilon), dev(wl.source), wl.omega,
                        wl.source_pos, wl.sim_params).cpu().numpy()
  want = _field_oracle(wl)
  assert got.shape == (1, 3) + wl.epsilon.shape[1:]
  assert np.array_equal(got, want.astype(np.complex64))


def test_field_c0_full_vs_fp32_and_fp64_oracle(native):
  """Config c0: 128x128x32, 2000 steps; bit-exact to the FP32 oracle and
  within 1e-5 relative L2 of the FP64 oracle."""
  wl = workloads.waveguide_c0()
  got = pjz_gb300.field(dev(wl.epsilon), dev(wl.source), wl.omega,
                        wl.source_pos, wl.sim_params).cpu().numpy()
  want32 = _field_oracle(wl, "f32")
  assert np.array_equal(got, want32.astype(np.complex64))
  want64 = _field_oracle(wl, "f64")
  err = np.linalg.norm(got - want64) / np.linalg.norm(want64)
  print(f"c0 FP32 engine vs FP64 oracle: rel-L2 {err:.3e}")
  assert err < 1e-5


@pytest.mark.parametrize("variant", VARIANTS, ids=VIDS)
def test_c1_size_short_run_bit_exact(native, variant):
  """Full 512x512x64 domain for 24 steps against the FP32 oracle."""
  wl = workloads.design_c1(tt=24, ww=5)
  sp = wl.sim_params
  kw, omega = pjz_ref.field_setup(wl.epsilon, wl.source, wl.omega, wl.source_pos,
                                  pjz_ref.SimParams(*sp[:-1]), zz=wl.domain[2])
  domain = wl.domain
  org, shp, prof = oracle.plane_source_box(kw["source_field"],
                                           kw["source_position"], domain)
  steps = (10, 24, 4)
  case = dict(eps=kw["epsilon"], offset=kw["offset"], mask=kw["absorption_mask"],
              kappa=kw["pml_kappa"], sigma=kw["pml_sigma"], alpha=kw["pml_alpha"],
              dt=0.5, tt=24, pml_widths=kw["pml_widths"], source_origin=org,
              source_profile=prof, waveform=kw["source_waveform"],
              output_steps=steps, domain=domain)
  want = oracle.run(**oracle_kwargs(case))["out"]
  got, _, _ = gpu_run(case, **variant)
  assert np.array_equal(got, want)


def test_linearity_at_full_size(native):
  """Doubling the source doubles every field (x2 is exact except where
  results are subnormal, so the check is to 1e-6 relative L2)."""
  wl = workloads.design_c1(tt=300, ww=2)
  a = pjz_gb300.field(dev(wl.epsilon), dev(wl.source), wl.omega, wl.source_pos,
                      wl.sim_params)
  b = pjz_gb300.field(dev(wl.epsilon), dev(2 * wl.source), wl.omega,
                      wl.source_pos, wl.sim_params)
  assert torch.isfinite(torch.view_as_real(a)).all()
  err = (torch.linalg.vector_norm(2 * a - b) / torch.linalg.vector_norm(b)).item()
  assert err < 1e-6, err
  c = pjz_gb300.field(dev(wl.epsilon), dev(wl.source), wl.omega, wl.source_pos,
                      wl.sim_params)
  assert torch.equal(a, c)  # deterministic


def test_cpu_tensor_inputs_are_rejected_by_plan(native):
  case = random_problem(10)
  p = engine.Plan(domain=case["domain"], offset=case["offset"],
                  region=case["eps"].shape[1:], tt=case["tt"], dt=0.5,
                  pml_widths=case["pml_widths"], pml_kappa=case["kappa"],
                  pml_sigma=case["sigma"], pml_alpha=case["alpha"])
  with pytest.raises(ValueError, match="CUDA"):
    p.run(epsilon=torch.as_tensor(case["eps"]),
          absorption_mask=torch.as_tensor(case["mask"]))
  with pytest.raises(ValueError, match="epsilon must have shape"):
    p.run(epsilon=dev(case["eps"][:, :-1]), absorption_mask=dev(case["mask"]))
