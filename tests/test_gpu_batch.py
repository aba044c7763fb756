"""Monitors and the batched scheduler: results must equal single-plan runs
(which equal the CPU oracle) bit for bit."""

import numpy as np
import pytest
import torch

import oracle
from pjz_gb300 import engine
from _cases import oracle_kwargs, random_problem

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def dev(a):
  return torch.as_tensor(np.ascontiguousarray(a), device=DEV)


def plan_of(case, out_mode=engine.OUT_SNAPSHOTS, weights=None, monitors=None,
            **kw):
  return engine.Plan(domain=case["domain"], offset=case["offset"],
                     region=case["eps"].shape[1:], tt=case["tt"], dt=case["dt"],
                     pml_widths=case["pml_widths"], pml_kappa=case["kappa"],
                     pml_sigma=case["sigma"], pml_alpha=case["alpha"],
                     source_origin=case["source_origin"],
                     source_shape=case["source_profile"].shape[2:],
                     source_ncols=case["source_profile"].shape[0],
                     output_steps=case["output_steps"], out_mode=out_mode,
                     weights=weights, monitors=monitors, **kw)


def inputs_of(case):
  return dict(epsilon=dev(case["eps"]), absorption_mask=dev(case["mask"]),
              source=dev(case["source_profile"]), waveform=dev(case["waveform"]))


@pytest.mark.parametrize("mode", [engine.OUT_SNAPSHOTS, engine.OUT_PHASORS])
def test_monitors_equal_region_slices(native, mode):
  case = random_problem(30, X=28, Y=24, Z=16, tt=50, steps=(20, 50, 6))
  ns = len(range(*case["output_steps"]))
  w = np.random.default_rng(1).normal(size=(4, ns)).astype(np.float32)
  wts = w if mode == engine.OUT_PHASORS else None
  full = plan_of(case, mode, wts)
  ref, _ = full.run(**inputs_of(case))
  boxes = [((3, 4, 2), (5, 6, 7)), ((20, 2, 5), (1, 20, 9)), ((2, 2, 2), (24, 20, 12))]
  mon = plan_of(case, mode, wts, monitors=boxes)
  out, _ = mon.run(**inputs_of(case))
  torch.cuda.synchronize()
  ox, oy, oz = case["offset"]
  for (o, s), v in zip(boxes, mon.split(out)):
    sl = (slice(None), slice(None), slice(o[0] - ox, o[0] - ox + s[0]),
          slice(o[1] - oy, o[1] - oy + s[1]), slice(o[2] - oz, o[2] - oz + s[2]))
    assert torch.equal(v, ref[sl])


def _mixed_cases():
  specs = [dict(X=26, Y=22, Z=16, tt=40, src="x", steps=(20, 40, 5)),
           dict(X=30, Y=18, Z=24, tt=56, src="y", src_pos=6, steps=(30, 56, 7)),
           dict(X=20, Y=28, Z=32, tt=48, src="z", src_pos=9, steps=(10, 48, 4)),
           dict(X=34, Y=30, Z=20, tt=60, src="x", steps=(40, 60, 3))]
  return [random_problem(40 + i, **s) for i, s in enumerate(specs)]


@pytest.mark.parametrize("spp", ["1", "2", "mixed"])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_equals_single_runs(native, graph, spp):
  """Uneven problems in one batch -- one step per launch, two, or a mix --
  equal their single-plan runs bit for bit (and the oracle)."""
  cases = _mixed_cases()
  plans, refs, ins = [], [], []
  for k, case in enumerate(cases):
    ns = len(range(*case["output_steps"]))
    knob = dict(steps_per_pass=int(spp) if spp != "mixed" else 1 + k % 2)
    if k % 2:
      w = np.random.default_rng(k).normal(size=(6, ns)).astype(np.float32)
      p = plan_of(case, engine.OUT_PHASORS, w, **knob)
    else:
      p = plan_of(case, **knob)
    assert p.launch_config()["steps_per_pass"] == knob["steps_per_pass"]
    ref, _ = p.run(**inputs_of(case))
    plans.append(p)
    refs.append(ref)
    ins.append(inputs_of(case))
  torch.cuda.synchronize()
  batch = engine.Batch(plans)
  outs = [torch.full_like(r, float("nan")) for r in refs]
  for _ in range(2 if graph else 1):  # second call replays the graph
    for o in outs:
      o.fill_(float("nan"))
    res = batch.run([dict(i, out=o) for i, o in zip(ins, outs)], graph=graph)
    torch.cuda.synchronize()
    batch.check_status()
    for (got, _), ref in zip(res, refs):
      assert torch.equal(got, ref)
  want = oracle.run(**oracle_kwargs(cases[0]))["out"]
  assert np.array_equal(outs[0].cpu().numpy(), want)


def test_batch_rejects_register_kernel_plans(native):
  case = random_problem(50, Z=18, pml=(3, 2))
  with pytest.raises(NotImplementedError, match="streamed"):
    engine.Batch([plan_of(case)])
