"""Plan/run wrapper over the pjzfdtd C ABI, with torch tensors as buffers.

A :class:`Plan` is the static part of one FDTD problem (domain, region,
source box, output schedule, z-PML coefficients, projection weights and
launch geometry), mirroring what pjz marks static when it jits ``field``
(``src/pjz/_field.py:171``).  Running it takes the dynamic device arrays
(epsilon, absorber, source, waveform) and writes the outputs, stream-ordered
on torch's current stream.  PyTorch only supplies device memory and the
stream; all compute is the native sm_103a library.
"""

import ctypes
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib

OUT_NONE = _lib.OUT_NONE
OUT_SNAPSHOTS = _lib.OUT_SNAPSHOTS
OUT_PHASORS = _lib.OUT_PHASORS
OUT_GRADIENT = _lib.OUT_GRADIENT
STORAGE_F32 = _lib.STORAGE_F32
STORAGE_F16 = _lib.STORAGE_F16


def _f32_host(a) -> np.ndarray:
  if isinstance(a, torch.Tensor):
    a = a.detach().cpu().numpy()
  return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _ptr(t: Optional[torch.Tensor]):
  return None if t is None else ctypes.c_void_p(t.data_ptr())


def _dev_f32(name: str, t, device, shape=None) -> torch.Tensor:
  if not isinstance(t, torch.Tensor):
    t = torch.as_tensor(np.asarray(t, dtype=np.float32))
  if t.dtype != torch.float32:
    t = t.to(torch.float32)
  t = t.to(device).contiguous()
  if shape is not None and tuple(t.shape) != tuple(shape):
    raise ValueError(f"{name} must have shape {tuple(shape)}, got {tuple(t.shape)}")
  return t


class Plan:
  """One FDTD problem's static configuration plus its device workspace."""

  def __init__(self, *, domain: Tuple[int, int, int],
               offset: Tuple[int, int, int], region: Tuple[int, int, int],
               tt: int, dt: float, pml_widths: Tuple[int, int], pml_kappa,
               pml_sigma, pml_alpha,
               source_origin: Tuple[int, int, int] = (0, 0, 0),
               source_shape: Tuple[int, int, int] = (0, 0, 0),
               source_ncols: int = 0,
               output_steps: Tuple[int, int, int] = (0, 0, 1),
               out_mode: int = OUT_NONE, weights=None, record_h: bool = False,
               grad_origin: Tuple[int, int, int] = (0, 0, 0),
               grad_shape: Tuple[int, int, int] = (0, 0, 0),
               tile_y: int = 0, seg_x: int = 0, steps_per_pass: int = 0,
               kernel: int = 0, stages: int = 0, monitors=None, warps: int = 0,
               wait_limit_kcycles: int = 0, test_stall_bytes: int = 0,
               storage: int = STORAGE_F32):
    lib = _lib.load()
    p = _lib.Problem()
    p.xx, p.yy, p.zz = (int(v) for v in domain)
    p.ox, p.oy, p.oz = (int(v) for v in offset)
    p.rx, p.ry, p.rz = (int(v) for v in region)
    p.tt = int(tt)
    p.pml_lo, p.pml_hi = (int(v) for v in pml_widths)
    p.dt = float(dt)
    p.src_x0, p.src_y0, p.src_z0 = (int(v) for v in source_origin)
    p.src_nx, p.src_ny, p.src_nz = (int(v) for v in source_shape)
    p.src_ncols = int(source_ncols)
    p.out_start, p.out_stop, p.out_step = (int(v) for v in output_steps)
    p.out_mode = int(out_mode)
    p.record_h = int(bool(record_h))
    p.grad_x0, p.grad_y0, p.grad_z0 = (int(v) for v in grad_origin)
    p.grad_nx, p.grad_ny, p.grad_nz = (int(v) for v in grad_shape)
    p.tile_y, p.seg_x, p.steps_per_pass = int(tile_y), int(seg_x), int(steps_per_pass)
    p.kernel, p.stages, p.warps = int(kernel), int(stages), int(warps)
    p.wait_limit_kcycles = int(wait_limit_kcycles)
    p.test_stall_bytes = int(test_stall_bytes)
    p.storage = int(storage)
    zz = p.zz
    kap, sig, alp = (_f32_host(a) for a in (pml_kappa, pml_sigma, pml_alpha))
    for name, a in (("pml_kappa", kap), ("pml_sigma", sig), ("pml_alpha", alp)):
      if a.shape != (zz, 2):
        raise ValueError(f"{name} must have shape ({zz}, 2), got {a.shape}")
    w = None
    if out_mode in (OUT_PHASORS, OUT_GRADIENT):
      w = _f32_host(weights)
      if w.ndim != 2:
        raise ValueError("weights must be (rows, ns)")
      p.out_rows = w.shape[0]
    self._keep = (kap, sig, alp, w)
    handle = ctypes.c_void_p()
    wp = None if w is None else w.ctypes.data
    _lib.check(lib.pjzfdtd_plan_create(ctypes.byref(p), kap.ctypes.data,
                                       sig.ctypes.data, alp.ctypes.data, wp,
                                       ctypes.byref(handle)))
    self._lib = lib
    self._h = handle
    self.problem = p
    nb = ctypes.c_size_t()
    _lib.check(lib.pjzfdtd_plan_workspace_bytes(handle, ctypes.byref(nb)))
    self.workspace_bytes = nb.value
    ns = ctypes.c_int32()
    _lib.check(lib.pjzfdtd_plan_num_samples(handle, ctypes.byref(ns)))
    self.num_samples = ns.value
    self._ws = None
    if w is not None and w.shape[1] != self.num_samples:
      raise ValueError(f"weights must have {self.num_samples} columns")
    self.monitors = None
    if monitors:
      self.set_monitors(monitors)

  def set_monitors(self, boxes):
    """Records only ``boxes`` (list of (origin, shape) in domain cells);
    ``out`` becomes flat, see :meth:`split`."""
    arr = np.ascontiguousarray(
        [[*map(int, o), *map(int, s)] for o, s in boxes], dtype=np.int32)
    _lib.check(self._lib.pjzfdtd_plan_set_monitors(self._h, len(boxes),
                                                   arr.ctypes.data))
    self.monitors = [(tuple(map(int, o)), tuple(map(int, s))) for o, s in boxes]
    nb = ctypes.c_size_t()
    _lib.check(self._lib.pjzfdtd_plan_workspace_bytes(self._h, ctypes.byref(nb)))
    self.workspace_bytes = nb.value
    self._ws = None

  def split(self, out: torch.Tensor):
    """Per-monitor views of a flat ``out``: ``(lead, 3, nx, ny, nz)`` each,
    ``lead`` = samples (snapshots) or weight rows (phasors)."""
    p = self.problem
    lead = self.num_samples if p.out_mode == OUT_SNAPSHOTS else p.out_rows
    views, o = [], 0
    for _, s in self.monitors:
      n = lead * 3 * s[0] * s[1] * s[2]
      views.append(out[o:o + n].view(lead, 3, *s))
      o += n
    return views

  def __del__(self):
    h = getattr(self, "_h", None)
    if h is not None and h.value:
      self._lib.pjzfdtd_plan_destroy(h)
      self._h = None

  # -- shapes ---------------------------------------------------------------
  @property
  def domain(self):
    p = self.problem
    return (p.xx, p.yy, p.zz)

  @property
  def region(self):
    p = self.problem
    return (p.rx, p.ry, p.rz)

  def out_shape(self):
    p = self.problem
    if self.monitors:
      n = ctypes.c_size_t()
      _lib.check(self._lib.pjzfdtd_plan_output_floats(self._h, ctypes.byref(n)))
      return (n.value,)
    if p.out_mode == OUT_SNAPSHOTS:
      return (self.num_samples, 3) + self.region
    if p.out_mode == OUT_PHASORS:
      return (p.out_rows, 3) + self.region
    if p.out_mode == OUT_GRADIENT:
      return (3, p.grad_nx, p.grad_ny, p.grad_nz)
    return None

  def launch_config(self):
    vals = [ctypes.c_int32() for _ in range(6)]
    _lib.check(self._lib.pjzfdtd_plan_launch_config(
        self._h, *(ctypes.byref(v) for v in vals)))
    return dict(zip(("tile_y", "seg_x", "threads", "steps_per_pass", "kernel",
                     "stages"), (v.value for v in vals)))

  def step_launches(self, n0: int = 0, n1: int = None) -> int:
    """Step-kernel launches for steps [n0, n1): the engine runs two steps
    per launch when the plan has two steps per pass and the state between
    them is not sampled, one step otherwise (the schedule of the C
    library's run loop)."""
    p = self.problem
    n1 = p.tt if n1 is None else n1
    two = self.launch_config()["steps_per_pass"] == 2
    sampled = lambda n: (p.out_mode != OUT_NONE and p.out_start <= n < p.out_stop
                         and (n - p.out_start) % p.out_step == 0)
    count, n = 0, n0
    while n < n1:
      n += 2 if (two and n + 1 < n1 and not sampled(n)) else 1
      count += 1
    return count

  def check_status(self, device=None):
    """Raises TimeoutError if a bounded device-side wait of the work queued
    so far gave up (synchronises torch's current stream)."""
    if self._ws is None:
      return
    dev = device or self._ws.device
    with torch.cuda.device(dev):
      stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
      _lib.check(self._lib.pjzfdtd_plan_status(
          self._h, ctypes.c_void_p(self._ws.data_ptr()), self._ws.numel(),
          stream))

  def workspace(self, device) -> torch.Tensor:
    if self._ws is None or self._ws.device != torch.device(device):
      self._ws = torch.empty(max(self.workspace_bytes, 256), dtype=torch.uint8,
                             device=device)
    return self._ws

  # -- execution ------------------------------------------------------------
  def buffers(self, *, epsilon, absorption_mask, source=None, waveform=None,
              q=None, out=None, out_h=None, fields=None):
    """Validates the device arrays of one run and allocates missing outputs;
    returns ``(pjzfdtd_buffers, keep-alive tensors, out, out_h)``."""
    p = self.problem
    dev = epsilon.device if isinstance(epsilon, torch.Tensor) else torch.device("cuda")
    if dev.type != "cuda":
      raise ValueError("pjz_gb300 runs on CUDA devices only; epsilon is on "
                       f"{dev}")
    eps = _dev_f32("epsilon", epsilon, dev, (3,) + self.region)
    mask = _dev_f32("absorption_mask", absorption_mask, dev, (3, p.xx, p.yy))
    src = wave = qq = None
    if p.src_ncols > 0:
      src = _dev_f32("source", source, dev,
                     (p.src_ncols, 3, p.src_nx, p.src_ny, p.src_nz))
      wave = _dev_f32("waveform", waveform, dev, (p.tt, p.src_ncols))
    if p.out_mode == OUT_GRADIENT:
      qq = _dev_f32("q", q, dev, (p.out_rows, 3, p.grad_nx, p.grad_ny, p.grad_nz))
    shape = self.out_shape()
    if shape is not None and out is None:
      out = torch.empty(shape, dtype=torch.float32, device=dev)
    if p.record_h and out_h is None:
      out_h = torch.empty(shape, dtype=torch.float32, device=dev)
    for name, t in (("out", out), ("out_h", out_h)):
      if t is not None and (t.dtype != torch.float32 or not t.is_contiguous()
                            or tuple(t.shape) != tuple(shape) or t.device != dev):
        raise ValueError(f"{name} must be a contiguous float32 {shape} tensor "
                         f"on {dev}")
    if fields is not None:
      if (fields.dtype != torch.float32 or not fields.is_contiguous()
          or tuple(fields.shape) != (6,) + self.domain or fields.device != dev):
        raise ValueError(f"fields must be a contiguous float32 {(6,) + self.domain}"
                         f" tensor on {dev}")
    b = _lib.Buffers(epsilon=_ptr(eps), absorption_mask=_ptr(mask),
                     source=_ptr(src), waveform=_ptr(wave), q=_ptr(qq),
                     out=_ptr(out), out_h=_ptr(out_h), fields=_ptr(fields))
    keep = (eps, mask, src, wave, qq, out, out_h, fields)
    return b, keep, out, out_h

  def run(self, *, epsilon, absorption_mask, source=None, waveform=None,
          q=None, out=None, out_h=None, fields=None, steps=None,
          workspace: Optional[torch.Tensor] = None):
    """Runs the plan; returns ``(out, out_h)`` (``out_h`` None unless H)."""
    p = self.problem
    b, keep, out, out_h = self.buffers(
        epsilon=epsilon, absorption_mask=absorption_mask, source=source,
        waveform=waveform, q=q, out=out, out_h=out_h, fields=fields)
    dev = keep[0].device
    ws = workspace if workspace is not None else self.workspace(dev)
    with torch.cuda.device(dev):
      stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
      ws_ptr = ctypes.c_void_p(ws.data_ptr())
      nbytes = ws.numel()
      if steps is not None:
        rc = self._lib.pjzfdtd_run_steps(self._h, ctypes.byref(b), ws_ptr,
                                         nbytes, int(steps[0]), int(steps[1]),
                                         stream)
      elif p.out_mode == OUT_GRADIENT:
        rc = self._lib.pjzfdtd_adjoint(self._h, ctypes.byref(b), ws_ptr,
                                       nbytes, stream)
      else:
        rc = self._lib.pjzfdtd_forward(self._h, ctypes.byref(b), ws_ptr,
                                       nbytes, stream)
    _lib.check(rc)
    return out, out_h


def plane_source_box(source_field: torch.Tensor, source_position: int,
                     domain: Sequence[int]):
  """Maps an fdtdz plane source onto the engine's source box.

  ``(2, 1, Y, Z)`` x-normal / ``(2, X, 1, Z)`` y-normal: waveform column 0
  drives plane ``source_position`` and column 1 plane ``source_position - 1``
  (what pjz relies on when it bumps odd positions and flips the columns,
  ``src/pjz/_field.py:230-233``); the two entries feed the two transverse E
  components in xyz order.  ``(2, 2, X, Y, 1)`` z-normal: column k carries
  profile ``source_field[k]`` on (Ex, Ey) at plane ``source_position``
  (``src/pjz/_field.py:234-236``).  Returns (origin, shape, profile).
  """
  X, Y, Z = (int(v) for v in domain)
  sf = source_field
  s = int(source_position)
  dev = sf.device
  if sf.dim() == 5:
    if tuple(sf.shape) != (2, 2, X, Y, 1):
      raise ValueError(f"z-normal source_field must be (2, 2, {X}, {Y}, 1), "
                       f"got {tuple(sf.shape)}")
    if not 0 <= s < Z:
      raise ValueError(f"source_position {s} outside [0, {Z})")
    prof = torch.zeros((2, 3, X, Y, 1), dtype=torch.float32, device=dev)
    prof[:, 0:2] = sf.to(torch.float32)
    return (0, 0, s), (X, Y, 1), prof
  if sf.dim() != 4 or sf.shape[0] != 2 or (sf.shape[1] != 1 and sf.shape[2] != 1):
    raise ValueError("source_field must be (2, 1, Y, Z), (2, X, 1, Z) or "
                     f"(2, 2, X, Y, 1), got {tuple(sf.shape)}")
  axis = 0 if sf.shape[1] == 1 else 1
  full = [X, Y, Z]
  expect = list(full)
  expect[axis] = 1
  if list(sf.shape[1:]) != expect:
    raise ValueError(f"source_field must be (2, {', '.join(map(str, expect))}), "
                     f"got {tuple(sf.shape)}")
  if not 0 <= s < full[axis]:
    raise ValueError(f"source_position {s} outside [0, {full[axis]})")
  comps = [c for c in range(3) if c != axis]
  lo = max(s - 1, 0)
  shape = list(full)
  shape[axis] = s + 1 - lo
  prof = torch.zeros((2, 3) + tuple(shape), dtype=torch.float32, device=dev)
  for col, plane in ((0, s), (1, s - 1)):
    if plane < 0:
      continue
    idx = [slice(None)] * 3
    idx[axis] = slice(plane - lo, plane - lo + 1)
    for k, c in enumerate(comps):
      prof[(col, c) + tuple(idx)] = sf[k].to(torch.float32)
  origin = [0, 0, 0]
  origin[axis] = lo
  return tuple(origin), tuple(shape), prof


def run_many(plans, inputs):
  """Runs independent plans: as one :class:`Batch` (one launch per time step
  for all of them) when every plan stores FP32 and none asked for the lean
  kernel, else one after another (batches run FP32 storage on the streamed
  kernels).  Returns the ``(out, out_h)`` pairs."""
  if all(p.problem.storage == STORAGE_F32 and p.problem.kernel != 3 for p in plans):
    return Batch(plans).run(inputs, graph=False)
  return [p.run(**kw) for p, kw in zip(plans, inputs)]


class Batch:
  """Independent plans advanced together: one kernel launch per time step
  for all of them, the whole run captured once into a CUDA graph.

  ``run`` takes one dict of :meth:`Plan.run` arguments per plan and returns
  the ``(out, out_h)`` pairs.  Graph replays need the same output tensors
  and inputs each time, so pass ``out`` tensors to reuse a captured graph.
  """

  def __init__(self, plans):
    lib = _lib.load()
    self.plans = list(plans)
    arr = (ctypes.c_void_p * len(self.plans))(*[p._h.value for p in self.plans])
    h = ctypes.c_void_p()
    _lib.check(lib.pjzfdtd_batch_create(arr, len(self.plans), ctypes.byref(h)))
    self._lib, self._h = lib, h
    nb = ctypes.c_size_t()
    _lib.check(lib.pjzfdtd_batch_workspace_bytes(h, ctypes.byref(nb)))
    self.workspace_bytes = nb.value
    self._ws = None
    self._stream = None
    self._keep = None

  def __del__(self):
    h = getattr(self, "_h", None)
    if h is not None and h.value:
      self._lib.pjzfdtd_batch_destroy(h)
      self._h = None

  def run(self, inputs, graph: bool = True):
    if len(inputs) != len(self.plans):
      raise ValueError("one input dict per plan")
    bufs, keep, outs = [], [], []
    for plan, kw in zip(self.plans, inputs):
      b, k, out, out_h = plan.buffers(**kw)
      bufs.append(b)
      keep.append(k)
      outs.append((out, out_h))
    dev = keep[0][0].device
    if self._ws is None or self._ws.device != dev:
      self._ws = torch.empty(max(self.workspace_bytes, 256), dtype=torch.uint8,
                             device=dev)
    arr = (_lib.Buffers * len(bufs))(*bufs)
    cur = torch.cuda.current_stream(dev)
    if self._stream is None:
      self._stream = torch.cuda.Stream(device=dev)
    side = self._stream
    side.wait_stream(cur)
    with torch.cuda.device(dev), torch.cuda.stream(side):
      rc = self._lib.pjzfdtd_batch_run(
          self._h, arr, ctypes.c_void_p(self._ws.data_ptr()), self._ws.numel(),
          int(bool(graph)), ctypes.c_void_p(side.cuda_stream))
    _lib.check(rc)
    cur.wait_stream(side)
    for k in keep:
      for t in k:
        if t is not None:
          t.record_stream(side)
    self._keep = keep  # the captured graph refers to these buffers
    return outs

  def check_status(self):
    """Raises TimeoutError if a bounded device wait of any plan gave up."""
    for i, p in enumerate(self.plans):
      off = 0
      # Each plan's workspace sits at its 256-byte aligned offset.
      for q in self.plans[:i]:
        off = (off + q.workspace_bytes + 255) // 256 * 256
      with torch.cuda.device(self._ws.device):
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.check(self._lib.pjzfdtd_plan_status(
            p._h, ctypes.c_void_p(self._ws.data_ptr() + off), p.workspace_bytes,
            stream))
