"""The eager-torch CPU port of the update (``oracle/yee_torch.py``, timed by
the bench as a second CPU baseline) computes the oracle's fields: FP32
agreement with the C oracle's FP32 run and its FP32 error against the FP64
run, with absorber, odd-width z-PML slabs, an offset epsilon region and a
two-column source."""

import numpy as np

import oracle
from oracle import pjz_ref, yee_torch


def _problem(rng, pml):
  X, Y, Z, tt = 20, 18, 16, 60
  sig = pjz_ref.pml_sigma(pml, Z, 0.5, 1.3).astype(np.float32)
  return dict(eps=rng.uniform(1, 12, (3, X - 4, Y - 4, Z - 2)).astype(np.float32),
              offset=(2, 2, 1), mask=pjz_ref.absorption_mask(X, Y, 3, 0.05).astype(np.float32),
              kappa=np.ones_like(sig), sigma=sig, alpha=np.full_like(sig, 0.05),
              dt=0.5, tt=tt, pml_widths=pml, source_origin=(5, 0, 0),
              source_profile=rng.normal(size=(2, 3, 2, Y, Z)).astype(np.float32),
              waveform=rng.normal(size=(tt, 2)).astype(np.float32))


def test_torch_port_matches_the_oracle():
  for seed, pml in ((0, (4, 3)), (1, (0, 5)), (2, (0, 0))):
    kw = _problem(np.random.default_rng(seed), pml)
    X, Y = kw["mask"].shape[1:]
    Z = kw["kappa"].shape[0]
    f32 = oracle.run(**kw, precision="f32", mode="none",
                     fields=np.zeros((6, X, Y, Z), np.float32))["fields"]
    f64 = oracle.run(**kw, precision="f64", mode="none",
                     fields=np.zeros((6, X, Y, Z)))["fields"]
    got = yee_torch.run(**kw)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert np.linalg.norm(f64) > 0
    assert rel(got, f32) < 1e-6, (pml, rel(got, f32))
    assert rel(got, f64) < 1e-5, (pml, rel(got, f64))
