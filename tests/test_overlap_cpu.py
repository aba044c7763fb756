"""The two-plane mode overlap and forward/backward wave fit of ``scatter``
(``pjz_gb300/_scatter.py``, torch) against the oracle's NumPy restatement of
pjz's ``_overlap`` / ``_amplitudes`` (``src/pjz/_field.py:293-338``) on
random fields: x- and y-normal modes, forward, backward and at-plane
sampling, complex128 throughout."""

import numpy as np
import pytest
import torch

from oracle import pjz_ref
from pjz_gb300 import _scatter


@pytest.mark.parametrize("axis", [0, 1])
@pytest.mark.parametrize("is_fwd", [None, True, False])
def test_overlap_matches_pjz(axis, is_fwd):
  rng = np.random.default_rng(10 * axis + {None: 0, True: 1, False: 2}[is_fwd])
  ww, xx, yy, zz, pos = 3, 10, 8, 6, 4
  shape = (ww, 2, 1, yy, zz) if axis == 0 else (ww, 2, xx, 1, zz)
  mode = rng.normal(size=shape) + 1j * rng.normal(size=shape)
  out = (rng.normal(size=(ww, 3, xx, yy, zz))
         + 1j * rng.normal(size=(ww, 3, xx, yy, zz)))
  beta = rng.uniform(0.2, 0.6, ww)
  want = pjz_ref.overlap(mode, beta, pos, is_fwd, out)
  got = _scatter._overlap(torch.as_tensor(mode), torch.as_tensor(beta), pos,
                          is_fwd, torch.as_tensor(out)).numpy()
  assert want.shape == got.shape == (ww, 2)
  np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
