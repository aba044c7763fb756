"""Launch geometry and schedule on the host (plan creation makes no CUDA
call): the temporal-block depth a plan resolves to, the argument checks of
`steps_per_pass`, and the step-launch schedule -- two steps per launch
except where a sampled state sits between them."""

import numpy as np
import pytest

from pjz_gb300 import _build, _lib, engine
from _cases import random_problem


@pytest.fixture(scope="module")
def lib():
  _build.build()
  return _lib.load()


def plan(case, **kw):
  return engine.Plan(domain=case["domain"], offset=case["offset"],
                     region=case["eps"].shape[1:], tt=case["tt"], dt=case["dt"],
                     pml_widths=case["pml_widths"], pml_kappa=case["kappa"],
                     pml_sigma=case["sigma"], pml_alpha=case["alpha"],
                     source_origin=case["source_origin"],
                     source_shape=case["source_profile"].shape[2:],
                     source_ncols=case["source_profile"].shape[0],
                     output_steps=case["output_steps"],
                     out_mode=engine.OUT_SNAPSHOTS, **kw)


def expected_launches(tt, steps, two):
  sampled = set(n for n in range(*steps) if 0 <= n < tt)
  count, n = 0, 0
  while n < tt:
    n += 2 if (two and n + 1 < tt and n not in sampled) else 1
    count += 1
  return count


@pytest.mark.parametrize("tt,steps", [(48, (30, 48, 5)), (41, (-6, 41, 2)),
                                      (40, (0, 40, 1)), (9, (8, 9, 1))])
def test_two_step_schedule(lib, tt, steps):
  case = random_problem(1, Z=16, tt=tt, steps=steps)
  p = plan(case, kernel=2, steps_per_pass=2)
  assert p.launch_config()["steps_per_pass"] == 2
  assert p.step_launches() == expected_launches(tt, steps, True)
  # every step is run exactly once: pairs plus singles cover [0, tt)
  assert expected_launches(tt, steps, True) >= (tt + 1) // 2


def test_auto_depth_is_one_step_and_schedule_is_per_step(lib):
  case = random_problem(2, Z=16, tt=30, steps=(10, 30, 4))
  p = plan(case, kernel=2)
  assert p.launch_config()["steps_per_pass"] == 1
  assert p.step_launches() == 30
  assert p.step_launches(5, 17) == 12


def test_steps_per_pass_checks(lib):
  case = random_problem(3, Z=18, pml=(3, 2))
  with pytest.raises(NotImplementedError, match="two steps"):
    plan(case, kernel=1, steps_per_pass=2)
  case = random_problem(4, Z=16)
  with pytest.raises(ValueError, match="steps_per_pass"):
    plan(case, kernel=2, steps_per_pass=3)
