"""Device-side failure detection without a GPU fault.

Every wait of the streamed kernel is bounded.  The test hook
``test_stall_bytes`` makes the producer announce more bytes than it copies,
so no ring slot ever completes (a flag nothing sets): every wait must run
out after ``wait_limit_kcycles``, the kernel must return, the status word
must read TIMEOUT, and the context must stay usable.
"""

import time

import numpy as np
import pytest
import torch

import oracle
from pjz_gb300 import engine
from _cases import oracle_kwargs, random_problem

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _plan(case, **kw):
  return engine.Plan(domain=case["domain"], offset=case["offset"],
                     region=case["eps"].shape[1:], tt=case["tt"], dt=case["dt"],
                     pml_widths=case["pml_widths"], pml_kappa=case["kappa"],
                     pml_sigma=case["sigma"], pml_alpha=case["alpha"],
                     source_origin=case["source_origin"],
                     source_shape=case["source_profile"].shape[2:],
                     source_ncols=case["source_profile"].shape[0],
                     output_steps=case["output_steps"],
                     out_mode=engine.OUT_SNAPSHOTS, kernel=2, **kw)


def _inputs(case):
  t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=DEV)
  return dict(epsilon=t(case["eps"]), absorption_mask=t(case["mask"]),
              source=t(case["source_profile"]), waveform=t(case["waveform"]))


def test_stalled_ring_times_out_and_reports(native):
  case = random_problem(60, X=24, Y=20, Z=16, tt=3, steps=(0, 3, 1))
  stalled = _plan(case, wait_limit_kcycles=1000, test_stall_bytes=16)
  t0 = time.perf_counter()
  stalled.run(**_inputs(case))
  torch.cuda.synchronize()  # every CTA gave up and returned
  assert time.perf_counter() - t0 < 30
  with pytest.raises(TimeoutError, match="wait exceeded"):
    stalled.check_status()
  stalled.check_status()  # the word was cleared

  # The context is still usable: a healthy plan matches the oracle.
  case = random_problem(61, Z=16, tt=40, steps=(20, 40, 5))
  ok = _plan(case)
  out, _ = ok.run(**_inputs(case))
  torch.cuda.synchronize()
  ok.check_status()
  assert np.array_equal(out.cpu().numpy(), oracle.run(**oracle_kwargs(case))["out"])
