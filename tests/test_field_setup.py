"""Host-side set-up of ``field`` (pjz ``src/pjz/_field.py:193-269``) against
the oracle's restatement, on CPU tensors (no engine call)."""

import numpy as np
import pytest
import torch

import oracle
from oracle import pjz_ref
from pjz_gb300 import _field, engine
from pjz_gb300._fdtdz import LaunchParams


def _inputs(kind, rng, complex_src=False):
  xx, yy, zz = 14, 12, 10
  eps = rng.uniform(1.5, 5.0, (3, xx, yy, zz)).astype(np.float32)
  shape = {"x": (2, 1, yy, zz), "y": (2, xx, 1, zz), "z": (2, xx, yy, 1)}[kind]
  src = rng.normal(size=shape).astype(np.float32)
  if complex_src:
    src = src + 1j * rng.normal(size=shape).astype(np.float32)
  return eps, src


@pytest.mark.parametrize("kind,pos,complex_src", [
    ("x", 4, False), ("x", 5, False), ("y", 3, False), ("y", 6, False),
    ("z", 4, True), ("z", 5, False), ("x", 5, True)])
@pytest.mark.parametrize("batch", [False, True])
def test_setup_matches_oracle(kind, pos, complex_src, batch):
  rng = np.random.default_rng(hash((kind, pos, complex_src)) % 2**32)
  eps, src = _inputs(kind, rng, complex_src)
  omega = np.array([0.15, 0.17])
  sp = _field.SimParams(omega_range=(0.15, 0.17), tt=300, absorption_padding=3,
                        absorption_coeff=1e-3, pml_widths=(2, 3),
                        use_z_as_batch=batch, use_reduced_precision=False,
                        launch_params=LaunchParams(zz=16))
  sp_ref = pjz_ref.SimParams(*sp[:-1], launch_params=None)
  got, _ = _field._setup(torch.as_tensor(eps), torch.as_tensor(src), omega, pos, sp)
  want, _ = pjz_ref.field_setup(eps, src, omega, pos, sp_ref, zz=16)
  assert got["source_position"] == want["source_position"]
  assert got["offset"] == want["offset"]
  assert tuple(got["output_steps"]) == tuple(want["output_steps"])
  for k in ("source_field", "source_waveform", "absorption_mask"):
    np.testing.assert_allclose(np.asarray(got[k]), want[k], rtol=1e-6, atol=1e-7,
                               err_msg=k)
  for k in ("pml_kappa", "pml_sigma", "pml_alpha"):
    np.testing.assert_array_equal(got[k], want[k])


@pytest.mark.parametrize("shape,pos", [((2, 1, 9, 7), 4), ((2, 1, 9, 7), 0),
                                       ((2, 11, 1, 7), 5), ((2, 2, 11, 9, 1), 3)])
def test_plane_source_box_matches_oracle(shape, pos):
  rng = np.random.default_rng(0)
  sf = rng.normal(size=shape).astype(np.float32)
  domain = (11, 9, 7)
  o1, s1, p1 = engine.plane_source_box(torch.as_tensor(sf), pos, domain)
  o2, s2, p2 = oracle.plane_source_box(sf, pos, domain)
  assert tuple(o1) == tuple(o2) and tuple(s1) == tuple(s2)
  np.testing.assert_array_equal(p1.numpy(), p2)


def test_bad_source_shape_raises_value_error():
  with pytest.raises(ValueError, match="exactly one value"):
    _field._prop_axis(np.zeros((2, 3, 4, 5)))
  with pytest.raises(ValueError):
    engine.plane_source_box(torch.zeros(2, 3, 4, 5), 1, (3, 4, 5))


def test_projection_weights_match_pjz_pinv():
  omega = np.array([0.15, 0.16])
  steps = (100, 140, 9)
  np.testing.assert_allclose(_field.projection_weights(omega, steps, 0.5),
                             pjz_ref.projection_weights(omega, steps, 0.5))
