"""bench.py's reference arm (the CPU oracle on the host cores) on CPU: one
JSON line with the keys the bench contract asks for, for a single box and
for a prefix of the many-box workload's seeded box list."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.timeout(300)
@pytest.mark.parametrize("extra", [["--workload", "riemann1d"],
                                   ["--workload", "batch4096", "--nboxes", "3", "--cpu-threads", "2"]])
def test_reference_arm_json_line(extra):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "3", "--warmup", "3"] + extra,
                         cwd=ROOT, capture_output=True, text=True, timeout=280)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["unit"] == d["metric"] == "cell-updates/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["steps"] == 3 and d["warmup"] == 3
    if "--cpu-threads" in extra:
        assert d["cpu_baseline"]["cores"] == 2
    if "batch4096" in extra:
        assert d["config"]["boxes"] == 3 and d["config"]["cells"] > 0
