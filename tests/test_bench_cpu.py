"""The bench's reference arm runs on the host alone: one JSON line with the
keys the bench contract requires (impl, metric, value, unit, steps, warmup,
config, cpu_baseline, e2e with zero host-device bytes), on a short c0 run."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
  out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl",
                        "reference", "--workload", "c0", "--tt", "12", "--steps", "1",
                        "--warmup", "0", "--cpu-seconds", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
  assert out.returncode == 0, out.stderr[-2000:]
  lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
  assert len(lines) == 1, out.stdout
  d = json.loads(lines[0])
  for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup",
            "higher_is_better", "config", "cpu_baseline", "e2e", "dtype"):
    assert k in d, k
  assert d["impl"] == "reference" and d["value"] > 0
  assert d["config"]["workload"] and d["config"]["domain"] == [128, 128, 32]
  cb = d["cpu_baseline"]
  assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
  assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
  assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]


def test_committed_traffic_summaries_are_consistent():
  """The DRAM traffic figures the bench line reports come from committed
  ncu summaries: read + write per launch over the cells of a launch, and
  the two-step kernel moves fewer DRAM bytes per cell-update than the 60
  algorithmic bytes (temporal blocking)."""
  sys.path.insert(0, ROOT)
  import bench
  for name, steps in (("yee_stream_c1", 1), ("yee_lean_c1", 1), ("yee_lean2_c1", 2),
                      ("yee_lean_f16_ty14_c1", 1), ("yee_lean_f16_ty28_c1", 1)):
    bpc, d = bench._profile_traffic(name)
    assert bpc is not None, name
    total = d["dram_bytes_read_per_launch"] + d["dram_bytes_write_per_launch"]
    assert abs(total / d["cells_per_launch"] - bpc) < 0.01, name
    assert d.get("steps_per_launch", 1) == steps, name
    per_update = bpc / steps
    limit = 30 * 1.2 if "f16" in name else 60 * 1.2
    assert per_update < limit, (name, per_update)
  assert bench._profile_traffic("yee_lean2_c1")[0] / 2 < bench.BYTES_PER_CELL
