"""The tangent-linear recipe of ``pjz_gb300/_tangent.py`` checked on the CPU
with the FP64 oracle: a permittivity voxel's derivative equals one more
solve from a zero state driven at that voxel by the current
``(E^{n+1} - E^n) / dt`` of the forward solve.  Against central differences
of the FP64 oracle forward (step 2^-14, exact in the FP32 input), the
projected phasors agree to 1e-6 relative over the region."""

import numpy as np
import pytest

import oracle
from _cases import oracle_kwargs, random_problem


@pytest.mark.parametrize("voxel", [(1, 6, 7, 5), (0, 9, 4, 6), (2, 11, 12, 3)])
def test_tangent_solve_equals_fp64_central_differences(voxel):
  case = random_problem(41, X=24, Y=20, Z=16, tt=160, pml=(2, 2),
                        steps=(100, 160, 7))
  case["mask"] = np.zeros_like(case["mask"])  # keep the perturbation visible
  ns = len(range(*case["output_steps"]))
  w = np.random.default_rng(5).normal(size=(4, ns)).astype(np.float32)
  kw = oracle_kwargs(case)
  tt, dt = case["tt"], case["dt"]
  ox, oy, oz = case["offset"]
  c, x, y, z = voxel

  def proj(eps):
    return oracle.run(**dict(kw, eps=eps), mode="project", weights=w,
                      precision="f64")["out"]

  h = 2.0 ** -14
  ep, em = case["eps"].copy(), case["eps"].copy()
  ep[voxel] += h
  em[voxel] -= h
  fd = (proj(ep) - proj(em)) / (2 * h)

  snaps = oracle.run(**dict(kw, output_steps=(0, tt, 1)), mode="snapshot",
                     precision="f64")["out"]
  e = snaps[:, c, x, y, z]
  wave = ((e - np.concatenate([[0.0], e[:-1]])) / dt)[:, None]
  prof = np.zeros((1, 3, 1, 1, 1), np.float32)
  prof[0, c] = 1.0
  tl = oracle.run(**dict(kw, source_origin=(x + ox, y + oy, z + oz),
                         source_profile=prof, waveform=wave),
                  mode="project", weights=w, precision="f64")["out"]
  err = np.linalg.norm(tl - fd) / np.linalg.norm(fd)
  assert np.linalg.norm(fd) > 0
  print(f"tangent vs FP64 central differences: rel-L2 {err:.2e}")
  assert err < 1e-6, err
