"""The forward entry point that allocates nothing (pjzfdtd_forward_static).

Some callers cannot call cudaMalloc -- a host whose device memory belongs to
another runtime's pool, or a loop that must not risk the implicit device
synchronisation of cudaMalloc/cudaFree.  For them the library keeps a fixed
64 MiB scratch array on each device.  These tests call it through the C ABI
and check that two calls in a row give exactly what the workspace-based
pjzfdtd_forward gives (the parity tolerance of this suite is bit-exact),
that a plan needing more scratch than the array holds is refused, and that a
solve whose bounded device waits ran out reports TIMEOUT through
pjzfdtd_forward_static_status (the status word lives in the static array,
which the caller cannot address).  The file is named to be collected last.
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


def _plan(case, out_mode, weights=None, **kw):
  return engine.Plan(domain=case["domain"], offset=case["offset"],
                     region=case["eps"].shape[1:], tt=case["tt"], dt=case["dt"],
                     pml_widths=case["pml_widths"], pml_kappa=case["kappa"],
                     pml_sigma=case["sigma"], pml_alpha=case["alpha"],
                     source_origin=case["source_origin"],
                     source_shape=case["source_profile"].shape[2:],
                     source_ncols=case["source_profile"].shape[0],
                     output_steps=case["output_steps"], out_mode=out_mode,
                     weights=weights, **kw)


def _buffers(ins, out):
  ptr = lambda t: ctypes.c_void_p(t.data_ptr())
  return _lib.Buffers(epsilon=ptr(ins["epsilon"]),
                      absorption_mask=ptr(ins["absorption_mask"]),
                      source=ptr(ins["source"]), waveform=ptr(ins["waveform"]),
                      q=None, out=ptr(out), out_h=None, fields=None)


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
  for _ in range(2):
    out = torch.full_like(ref, float("nan"))
    b = _buffers(ins, out)
    _lib.check(native.pjzfdtd_forward_static(plan._h, ctypes.byref(b), stream))
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    _lib.check(native.pjzfdtd_forward_static_status(plan._h, stream))


def test_static_scratch_reports_a_wait_that_ran_out(native):
  """The test hook makes the producer announce 16 bytes more than it copies,
  so no ring slot completes and every bounded wait gives up (a flag nothing
  sets; no fault).  The static path must report it, clear it, and still
  give exact results on the next call."""
  case = random_problem(23, X=24, Y=20, Z=16, tt=3, steps=(0, 3, 1))
  stalled = _plan(case, engine.OUT_SNAPSHOTS, kernel=2,
                  wait_limit_kcycles=1000, test_stall_bytes=16)
  ins = dict(epsilon=_dev(case["eps"]), absorption_mask=_dev(case["mask"]),
             source=_dev(case["source_profile"]), waveform=_dev(case["waveform"]))
  out = torch.empty(stalled.out_shape(), device=DEV)
  stream = ctypes.c_void_p(torch.cuda.current_stream(DEV).cuda_stream)
  b = _buffers(ins, out)
  _lib.check(native.pjzfdtd_forward_static(stalled._h, ctypes.byref(b), stream))
  assert native.pjzfdtd_forward_static_status(stalled._h, stream) == _lib.ERR_TIMEOUT
  assert "wait exceeded" in _lib.last_error()
  _lib.check(native.pjzfdtd_forward_static_status(stalled._h, stream))  # cleared

  healthy = _plan(case, engine.OUT_SNAPSHOTS, kernel=2)
  ref, _ = healthy.run(**ins)
  out2 = torch.full_like(ref, float("nan"))
  b2 = _buffers(ins, out2)
  _lib.check(native.pjzfdtd_forward_static(healthy._h, ctypes.byref(b2), stream))
  _lib.check(native.pjzfdtd_forward_static_status(healthy._h, stream))
  torch.cuda.synchronize()
  assert torch.equal(out2, ref)


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
