"""ctypes binding of the pjzfdtd C ABI (``include/pjzfdtd.h``).

Loads the in-tree ``libpjzfdtd.so``; there is no fallback: if the library is
missing the import of the engine fails with an explicit error.
"""

import ctypes
import os

from . import _build

OK, ERR_INVALID, ERR_CUDA, ERR_WORKSPACE, ERR_TIMEOUT, ERR_UNSUPPORTED = range(6)
OUT_NONE, OUT_SNAPSHOTS, OUT_PHASORS, OUT_GRADIENT = range(4)
STORAGE_F32, STORAGE_F16 = range(2)
MAX_ROWS = 32

_PROBLEM_INTS = (
    "xx", "yy", "zz", "ox", "oy", "oz", "rx", "ry", "rz", "tt", "pml_lo",
    "pml_hi")
_PROBLEM_INTS2 = (
    "src_x0", "src_y0", "src_z0", "src_nx", "src_ny", "src_nz", "src_ncols",
    "out_start", "out_stop", "out_step", "out_mode", "out_rows", "record_h",
    "grad_x0", "grad_y0", "grad_z0", "grad_nx", "grad_ny", "grad_nz",
    "tile_y", "seg_x", "steps_per_pass", "kernel", "stages", "warps",
    "wait_limit_kcycles", "test_stall_bytes", "storage")


class Problem(ctypes.Structure):
  """Mirror of ``pjzfdtd_problem``."""
  _fields_ = ([(n, ctypes.c_int32) for n in _PROBLEM_INTS]
              + [("dt", ctypes.c_float)]
              + [(n, ctypes.c_int32) for n in _PROBLEM_INTS2])


class Buffers(ctypes.Structure):
  """Mirror of ``pjzfdtd_buffers`` (device pointers)."""
  _fields_ = [(n, ctypes.c_void_p) for n in (
      "epsilon", "absorption_mask", "source", "waveform", "q", "out", "out_h",
      "fields")]


# Every symbol include/pjzfdtd.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I = ctypes.c_int32
SIGNATURES = {
    "pjzfdtd_abi_version": (_I, []),
    "pjzfdtd_last_error": (_I, [ctypes.c_char_p, ctypes.c_size_t]),
    "pjzfdtd_plan_create": (_I, [ctypes.POINTER(Problem), _P, _P, _P, _P,
                                 ctypes.POINTER(_P)]),
    "pjzfdtd_plan_workspace_bytes": (_I, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "pjzfdtd_plan_num_samples": (_I, [_P, ctypes.POINTER(_I)]),
    "pjzfdtd_plan_destroy": (_I, [_P]),
    "pjzfdtd_forward": (_I, [_P, ctypes.POINTER(Buffers), _P, ctypes.c_size_t,
                             _P]),
    "pjzfdtd_adjoint": (_I, [_P, ctypes.POINTER(Buffers), _P, ctypes.c_size_t,
                             _P]),
    "pjzfdtd_run_steps": (_I, [_P, ctypes.POINTER(Buffers), _P,
                               ctypes.c_size_t, _I, _I, _P]),
    "pjzfdtd_plan_launch_config": (_I, [_P] + [ctypes.POINTER(_I)] * 6),
    "pjzfdtd_plan_status": (_I, [_P, _P, ctypes.c_size_t, _P]),
    "pjzfdtd_forward_static": (_I, [_P, ctypes.POINTER(Buffers), _P]),
    "pjzfdtd_forward_static_status": (_I, [_P, _P]),
    "pjzfdtd_plan_set_monitors": (_I, [_P, _I, _P]),
    "pjzfdtd_plan_output_floats": (_I, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "pjzfdtd_batch_create": (_I, [_P, _I, ctypes.POINTER(_P)]),
    "pjzfdtd_batch_workspace_bytes": (_I, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "pjzfdtd_batch_run": (_I, [_P, _P, _P, ctypes.c_size_t, _I, _P]),
    "pjzfdtd_batch_destroy": (_I, [_P]),
    "pjzfdtd_render_epsilon": (_I, [_P, _I, _I, _I, _I, _I, _P, _I, _P, _P]),
    "pjzfdtd_plane_overlaps": (_I, [_I, _P, _P, _P, _P, _I, _P, _P]),
    "pjzfdtd_smatrix_gradient": (_I, [_I, _I, ctypes.c_int64, _P, _P, _P, _P, _P,
                                      _P]),
}

_lib = None


class EngineError(RuntimeError):
  """A non-argument failure reported by the native engine."""


def load(path: str = None):
  """Loads (once) and returns the native library; raises if it is missing."""
  global _lib
  if _lib is not None:
    return _lib
  path = path or _build.LIB_PATH
  if not os.path.exists(path):
    raise ImportError(
        f"pjz_gb300 native library not found at {path}; build it with "
        "pjz_gb300._build.build() (nvcc, sm_103a). There is no CPU fallback.")
  lib = ctypes.CDLL(path)
  for name, (res, args) in SIGNATURES.items():
    fn = getattr(lib, name)
    fn.restype = res
    fn.argtypes = args
  _lib = lib
  return lib


def last_error() -> str:
  buf = ctypes.create_string_buffer(512)
  load().pjzfdtd_last_error(buf, len(buf))
  return buf.value.decode(errors="replace")


def check(rc: int) -> None:
  """Raises the Python exception matching a pjzfdtd status code."""
  if rc == OK:
    return
  msg = last_error()
  if rc == ERR_INVALID:
    raise ValueError(msg)
  if rc == ERR_UNSUPPORTED:
    raise NotImplementedError(msg)
  if rc == ERR_TIMEOUT:
    raise TimeoutError(msg)
  raise EngineError(f"pjzfdtd error {rc}: {msg}")
