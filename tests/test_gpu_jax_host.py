"""The bodies of the JAX shim's callbacks (``pjz_gb300/_jax_host.py``), which
need no jax: on host arrays they equal ``pjz_gb300.field`` and its torch
autograd backward bit for bit, with JAX's cotangent convention (the
conjugate of torch's) turned into torch's."""

import numpy as np
import pytest
import torch

import pjz_gb300
from pjz_gb300 import _jax_host
from test_gpu_adjoint import _small

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def test_field_host_equals_field(native):
  eps, src, omega, pos, sp, _ = _small(True, tt=600)
  got = _jax_host.field_host(eps, src, omega, pos, sp)
  want = pjz_gb300.field(torch.as_tensor(eps, device=DEV),
                         torch.as_tensor(src, device=DEV), omega, pos, sp)
  assert got.dtype == np.complex64
  assert np.array_equal(got, want.cpu().numpy())


def test_field_vjp_host_equals_torch_backward(native):
  eps, src, omega, pos, sp, c = _small(True, tt=600)
  # JAX's cotangent of L = Re(sum conj(c) F) is conj(c); torch's is c.
  got = _jax_host.field_vjp_host(eps, src, omega, np.conj(c), pos, sp)
  e = torch.tensor(eps, device=DEV, requires_grad=True)
  F = pjz_gb300.field(e, torch.as_tensor(src, device=DEV), omega, pos, sp)
  torch.real(torch.sum(torch.conj(torch.as_tensor(c, dtype=torch.complex64,
                                                  device=DEV)) * F)).backward()
  assert got.dtype == np.float32 and got.shape == eps.shape
  assert np.array_equal(got, e.grad.cpu().numpy())
