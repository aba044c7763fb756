"""Host logic of ``pjz_gb300.scatter`` (no GPU): the solves one call runs
(one per port with the frequency-averaged mode, as pjz does at
``src/pjz/_field.py:354-356``, or one per (port, frequency) with
``per_frequency``), the sample planes its overlaps read (the union over
ports, as ``_overlap`` picks them at ``src/pjz/_field.py:305-338``), and the
refusal of a plane outside the epsilon region."""

import numpy as np
import pytest
import torch

import pjz_gb300
from pjz_gb300 import _scatter


def _modes():
  m0 = torch.zeros((3, 2, 1, 6, 4), dtype=torch.complex64)
  m0[:, 0] = torch.arange(3, dtype=torch.float32)[:, None, None, None] + 1
  m1 = torch.zeros((3, 2, 5, 1, 4), dtype=torch.complex64)
  m1[:, 1] = 2.0
  return [m0, m1]


def test_solves_average_or_split_frequencies():
  sp = pjz_gb300.SimParams(omega_range=(0.1, 0.3), tt=100)
  omega = np.array([0.1, 0.2, 0.3])
  modes = _modes()
  avg = _scatter._solves(modes, (3, 2), omega, sp, False)
  assert [(i, k) for i, k, *_ in avg] == [(0, None), (1, None)]
  assert torch.equal(avg[0][2], modes[0].mean(dim=0))
  per = _scatter._solves(modes, (3, 2), omega, sp, True)
  assert [(i, k) for i, k, *_ in per] == [(i, k) for i in range(2) for k in range(3)]
  for i, k, src, p, om, spk in per:
    assert torch.equal(src, modes[i][k])
    assert om == [omega[k]] and spk.omega_range == (omega[k], omega[k])
    assert spk.tt == sp.tt and p == (3, 2)[i]


def test_sample_planes_union_and_bounds():
  modes = _modes()
  shape = (3, 8, 7, 4)
  planes = _scatter._planes(modes, (3, 2), (True, False), shape)
  assert planes == [(0, 4), (0, 5), (1, 0), (1, 1)]
  assert _scatter._planes(modes, (3, 2), (None, None), shape) == [(0, 3), (1, 2)]
  with pytest.raises(ValueError, match="outside the epsilon region"):
    _scatter._planes(modes, (6, 2), (True, None), shape)
  with pytest.raises(ValueError, match="outside the epsilon region"):
    _scatter._planes(modes, (3, 1), (True, False), shape)
