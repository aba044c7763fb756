"""Seeded random FDTD problems shared by the parity tests."""

import numpy as np

import oracle
from oracle import pjz_ref


def random_problem(seed, X=24, Y=20, Z=16, tt=48, pml=(2, 2), src="x",
                   src_pos=7, steps=(30, 48, 5), batch=False, alpha=0.05,
                   absorber=3, region_pad=(2, 2, 2)):
  rng = np.random.default_rng(seed)
  px, py, pz = region_pad
  eps = rng.uniform(1.5, 6.0, (3, X - 2 * px, Y - 2 * py, Z - 2 * pz)).astype(np.float32)
  mask = pjz_ref.absorption_mask(X, Y, absorber, 0.02).astype(np.float32)
  if batch:
    kap = np.full((Z, 2), np.inf, np.float32)
    sig = np.zeros((Z, 2), np.float32)
    alp = np.zeros((Z, 2), np.float32)
  else:
    sig = pjz_ref.pml_sigma(pml, Z, 0.5, 1.3).astype(np.float32)
    kap = np.ones_like(sig)
    alp = (alpha * np.ones_like(sig)).astype(np.float32)
  if src == "x":
    sf = rng.normal(size=(2, 1, Y, Z))
  elif src == "y":
    sf = rng.normal(size=(2, X, 1, Z))
  else:
    sf = rng.normal(size=(2, 2, X, Y, 1))
  sf = sf.astype(np.float32)
  org, shp, prof = oracle.plane_source_box(sf, src_pos, (X, Y, Z))
  wave = rng.normal(size=(tt, 2)).astype(np.float32)
  return dict(eps=eps, offset=region_pad, mask=mask, kappa=kap, sigma=sig,
              alpha=alp, dt=0.5, tt=tt, pml_widths=pml, source_origin=org,
              source_profile=prof, waveform=wave, output_steps=steps,
              source_field=sf, source_position=src_pos, domain=(X, Y, Z))


def oracle_kwargs(case):
  return {k: v for k, v in case.items()
          if k not in ("source_field", "source_position", "domain")}
