"""The autotuner's search space covers both temporal-block depths (one and
two time steps per HBM pass) with their tile and ring-depth axes."""

from pjz_gb300 import autotune


def test_candidates_cover_both_depths():
  cands = autotune.candidates((256, 256, 64), (8, 8))
  depths = {c["steps_per_pass"] for c in cands}
  assert depths == {1, 2}
  for spp in (1, 2):
    sub = [c for c in cands if c["steps_per_pass"] == spp]
    assert len({c["tile_y"] for c in sub}) > 1
    assert len({c["stages"] for c in sub}) > 1
  assert all(set(c) == {"steps_per_pass", "tile_y", "stages", "seg_mult"}
             for c in cands)
