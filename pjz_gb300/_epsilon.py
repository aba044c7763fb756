"""pjz's ``epsilon`` on the GPU.

``epsilon(layers, interface_positions, magnification, zz,
use_simple_averaging)`` keeps the signature and result of
``src/pjz/_epsilon.py:104-155``: the ``(3, xx, yy, zz)`` Yee-cell
permittivity of a layered stack of ``(ll, 2m*xx, 2m*yy)`` magnified
profiles with subpixel smoothing.  It runs the native kernel
(``csrc/render_kernel.cuh``) on torch's current stream, so a design ->
epsilon -> :func:`pjz_gb300.field` chain stays on the device.  Unlike pjz's
JAX version it is not differentiable.
"""

import ctypes

import numpy as np
import torch

from . import _lib


def epsilon(layers, interface_positions, magnification: int, zz: int,
            use_simple_averaging: bool = False, out: torch.Tensor = None):
  """Returns the ``(3, xx, yy, zz)`` float32 permittivity on the layers'
  CUDA device (``layers`` on the host are copied to the current device)."""
  lib = _lib.load()
  m = int(magnification)
  zz = int(zz)
  if m < 1 or zz < 1:
    raise ValueError(f"magnification and zz must be positive, got {m}, {zz}")
  t = torch.as_tensor(layers)
  if t.ndim != 3:
    raise ValueError(f"layers must be (ll, 2m*xx, 2m*yy), got {tuple(t.shape)}")
  ll, px, py = t.shape
  if px % (2 * m) or py % (2 * m) or px == 0 or py == 0:
    raise ValueError(f"layer profiles {px} x {py} are not whole cells of "
                     f"{2 * m} x {2 * m} pixels")
  xx, yy = px // (2 * m), py // (2 * m)
  pos = interface_positions
  if isinstance(pos, torch.Tensor):
    pos = pos.detach().cpu().numpy()
  pos = np.ascontiguousarray(np.asarray(pos, np.float32).reshape(-1))
  if pos.size != ll - 1:
    raise ValueError(f"{ll} layers need {ll - 1} interface positions, got "
                     f"{pos.size}")
  dev = t.device if t.is_cuda else torch.device("cuda", torch.cuda.current_device())
  t = t.to(device=dev, dtype=torch.float32).contiguous()
  shape = (3, xx, yy, zz)
  if out is None:
    out = torch.empty(shape, dtype=torch.float32, device=dev)
  elif (out.dtype != torch.float32 or not out.is_contiguous()
        or tuple(out.shape) != shape or out.device != dev):
    raise ValueError(f"out must be a contiguous float32 {shape} tensor on {dev}")
  with torch.cuda.device(dev):
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rc = lib.pjzfdtd_render_epsilon(
        ctypes.c_void_p(t.data_ptr()), ll, xx, yy, zz, m,
        ctypes.c_void_p(pos.ctypes.data) if pos.size else None,
        int(bool(use_simple_averaging)), ctypes.c_void_p(out.data_ptr()), stream)
  _lib.check(rc)
  return out
