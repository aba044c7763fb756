"""The forward entry point that allocates nothing (pjzfdtd_forward_static).

Some callers cannot call cudaMalloc -- a host whose device memory belongs to
another runtime's pool, or a loop that must not risk the implicit device
synchronisation of cudaMalloc/cudaFree.  For them the library keeps a fixed
64 MiB scratch array on each device.  These tests call it through the C ABI
and check that two calls in a row give exactly what the workspace-based
pjzfdtd_forward gives (the parity tolerance of this suite is bit-exact), and
that a plan needing more scratch than the array holds is refused.  The file
is named to be collected last.
"""

import ctypes

import numpy as np
import pytest
import torch

from pjz_gb300 import _lib, engine
from _cases import random_problem

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _dev(a):
  return torch.as_tensor(np.ascontiguousarray(a), device=DEV)


def _plan(case, out_mode, weights=None):
  return engine.Plan(domain=case["domain"], offset=case["offset"],
                     region=case["eps"].shape[1:], tt=case["tt"], dt=case["dt"],
                     pml_widths=case["pml_widths"], pml_kappa=case["kappa"],
                     pml_sigma=case["sigma"], pml_alpha=case["alpha"],
                     source_origin=case["source_origin"],
                     source_shape=case["source_profile"].shape[2:],
                     source_ncols=case["source_profile"].shape[0],
                     output_steps=case["output_steps"], out_mode=out_mode,
                     weights=weights)


@pytest.mark.parametrize("mode", ["snapshots", "phasors"])
def test_static_scratch_matches_workspace_forward_twice(native, mode):
  case = random_problem(21, X=40, Y=36, Z=32, tt=120, pml=(4, 4),
                        steps=(60, 120, 9))
  ns = len(range(*case["output_steps"]))
  if mode == "snapshots":
    plan = _plan(case, engine.OUT_SNAPSHOTS)
  else:
    w = np.random.default_rng(2).normal(size=(6, ns)).astype(np.float32)
    plan = _plan(case, engine.OUT_PHASORS, w)
  assert plan.workspace_bytes <= 64 << 20
  ins = dict(epsilon=_dev(case["eps"]), absorption_mask=_dev(case["mask"]),
             source=_dev(case["source_profile"]), waveform=_dev(case["waveform"]))
  ref, _ = plan.run(**ins)
  torch.cuda.synchronize()
  stream = ctypes.c_void_p(torch.cuda.current_stream(DEV).cuda_stream)
  ptr = lambda t: ctypes.c_void_p(t.data_ptr())
  for _ in range(2):
    out = torch.full_like(ref, float("nan"))
    b = _lib.Buffers(epsilon=ptr(ins["epsilon"]),
                     absorption_mask=ptr(ins["absorption_mask"]),
                     source=ptr(ins["source"]), waveform=ptr(ins["waveform"]),
                     q=None, out=ptr(out), out_h=None, fields=None)
    _lib.check(native.pjzfdtd_forward_static(plan._h, ctypes.byref(b), stream))
    torch.cuda.synchronize()
    assert torch.equal(out, ref)


def test_static_scratch_refuses_plans_beyond_its_size(native):
  case = random_problem(22, X=256, Y=256, Z=64, tt=4, pml=(8, 8), steps=(0, 4, 1),
                        region_pad=(0, 0, 0))
  plan = _plan(case, engine.OUT_SNAPSHOTS)
  assert plan.workspace_bytes > 64 << 20
  b = _lib.Buffers()
  stream = ctypes.c_void_p(torch.cuda.current_stream(DEV).cuda_stream)
  rc = native.pjzfdtd_forward_static(plan._h, ctypes.byref(b), stream)
  assert rc == _lib.ERR_WORKSPACE
  assert "64 MiB" in _lib.last_error()
