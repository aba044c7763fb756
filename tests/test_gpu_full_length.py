"""The benchmarked configurations at full length against the CPU oracle.

* c1 exactly as ``bench.py`` times it: the 512x512x64 domain, 10000 steps,
  5 frequencies over 1.50-1.60 um, phasors projected at the sample steps,
  through ``pjz_gb300.field``.  The GPU result must equal the FP32 oracle
  bit for bit (same IEEE operations in the same order, including the
  Kahan-compensated projection), and stay within 1e-5 relative L2 of the
  FP64 oracle over all five frequencies and three components (the field
  gate of the forward solve).  Both oracle legs run the C restatement on
  every host core; their times are printed.  The same solve with binary16
  storage (use_reduced_precision=True) is held to 2e-2 of the FP64 oracle
  and its error printed.
* c3 shapes in one graph-captured batch: several of c3's uneven problems
  (x, y in {256, 384, 512}, z in {32, 48, 64}, 1-3 frequencies, their own
  designs and source planes) for 240 steps each, every problem's phasors
  bit-equal to its FP32 oracle run.
"""

import time

import numpy as np
import pytest
import torch

import oracle
import pjz_gb300
from oracle import pjz_ref
from pjz_gb300 import _field, engine, workloads
from _cases import field_oracle

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def dev(a):
  return torch.as_tensor(np.ascontiguousarray(a), device=DEV)


def c3_pick(wls, n=6):
  """The first problem of each z extent (32, 48, 64), then further problems
  of new (x, y, z) shapes, up to ``n``: three z extents, several x / y sizes
  and 1-3 frequencies."""
  pick, seen = [], set()
  for z in (32, 48, 64):
    wl = next(w for w in wls if w.domain[2] == z)
    pick.append(wl)
    seen.add(wl.domain)
  for wl in wls:
    if len(pick) < n and wl.domain not in seen:
      seen.add(wl.domain)
      pick.append(wl)
  return pick


def test_c1_full_length_vs_fp32_and_fp64_oracle(native):
  wl = workloads.design_c1()
  assert wl.domain == (512, 512, 64) and wl.sim_params.tt == 10000
  assert len(wl.omega) == 5
  t0 = time.perf_counter()
  got = pjz_gb300.field(dev(wl.epsilon), dev(wl.source), wl.omega,
                        wl.source_pos, wl.sim_params).cpu().numpy()
  t_gpu = time.perf_counter() - t0
  assert np.isfinite(got.view(np.float32)).all()
  t0 = time.perf_counter()
  want32 = field_oracle(wl, "f32").astype(np.complex64)
  t32 = time.perf_counter() - t0
  same = np.array_equal(got, want32)
  t0 = time.perf_counter()
  want64 = field_oracle(wl, "f64")
  t64 = time.perf_counter() - t0
  err = np.linalg.norm(got - want64) / np.linalg.norm(want64)
  per_freq = [np.linalg.norm(got[k] - want64[k]) / np.linalg.norm(want64[k])
              for k in range(got.shape[0])]
  print(f"\nc1 full length (512x512x64, 10000 steps, 5 freqs): GPU {t_gpu:.1f} s "
        f"(incl. set-up and copies), FP32 oracle {t32:.1f} s, FP64 oracle "
        f"{t64:.1f} s; bit-exact to FP32 oracle: {same}; rel-L2 vs FP64 "
        f"{err:.3e} (per frequency {', '.join(f'{e:.2e}' for e in per_freq)})")
  sp16 = wl.sim_params._replace(use_reduced_precision=True)
  got16 = pjz_gb300.field(dev(wl.epsilon), dev(wl.source), wl.omega,
                          wl.source_pos, sp16).cpu().numpy()
  err16 = np.linalg.norm(got16 - want64) / np.linalg.norm(want64)
  print(f"c1 full length with binary16 storage: rel-L2 vs FP64 {err16:.3e}")
  assert same, np.abs(got - want32).max()
  assert err < 1e-5, err
  assert err16 < 2e-2, err16


def test_c3_shapes_batched_vs_oracle(native):
  pick = c3_pick(workloads.batch_c3(n=64, tt=240))
  plans, ins, refs = [], [], []
  for wl in pick:
    eps = dev(wl.epsilon)
    kw, om = _field._setup(eps, dev(wl.source), wl.omega, wl.source_pos,
                           wl.sim_params)
    plan, prof = _field.phasor_plan(kw, om)
    plans.append(plan)
    ins.append(dict(epsilon=eps, absorption_mask=kw["absorption_mask"],
                    source=prof, waveform=kw["source_waveform"],
                    out=torch.full(plan.out_shape(), float("nan"), device=DEV)))
  batch = engine.Batch(plans)
  res = batch.run(ins, graph=True)
  torch.cuda.synchronize()
  batch.check_status()
  for wl, plan, (out, _) in zip(pick, plans, res):
    ww = len(wl.omega)
    r = out.cpu().numpy()
    got = r[:ww] + 1j * r[ww:]
    want = field_oracle(wl, "f32")
    assert np.array_equal(got.astype(np.complex64), want.astype(np.complex64)), \
        (wl.name, np.abs(got - want).max())
