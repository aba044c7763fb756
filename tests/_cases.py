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


def field_oracle(wl, precision="f32", nthreads=0, storage="f32"):
  """pjz's ``field`` of workload ``wl`` on the CPU oracle: the restated
  pre-processing (``oracle/pjz_ref.py``), the C Yee update in FP32 or FP64
  and the pinv projection accumulated at the sample steps; returns the
  complex ``(ww, 3, xx, yy, zz)`` fields."""
  kw, omega = pjz_ref.field_setup(wl.epsilon, wl.source, wl.omega, wl.source_pos,
                                  pjz_ref.SimParams(*wl.sim_params[:-1]),
                                  zz=wl.domain[2])
  domain = (kw["absorption_mask"].shape[1], kw["absorption_mask"].shape[2],
            kw["pml_kappa"].shape[0])
  org, shp, prof = oracle.plane_source_box(kw["source_field"],
                                           kw["source_position"], domain)
  w = pjz_ref.projection_weights(omega, kw["output_steps"], kw["dt"])
  r = oracle.run(eps=kw["epsilon"], offset=kw["offset"],
                 mask=kw["absorption_mask"], kappa=kw["pml_kappa"],
                 sigma=kw["pml_sigma"], alpha=kw["pml_alpha"], dt=kw["dt"],
                 tt=kw["source_waveform"].shape[0], pml_widths=kw["pml_widths"],
                 source_origin=org, source_profile=prof,
                 waveform=kw["source_waveform"], output_steps=kw["output_steps"],
                 mode="project", weights=w, precision=precision,
                 nthreads=nthreads, storage=storage)["out"]
  ww = omega.shape[0]
  return r[:ww] + 1j * r[ww:]
