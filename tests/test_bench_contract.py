"""bench.py's reference arm on the CPU: one JSON line on the same metric,
unit and workload as the GPU arm, with impl "reference", a cpu_baseline that
describes the run and an e2e object with no host-device bytes; the steps it
reports are the steps it timed, on the mesh size it reports."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "2", "--warmup", "1", "--n", "17"], cwd=ROOT,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["steps"] == 2 and d["warmup"] == 1
    assert d["config"]["nodes"] == 17 ** 3 and d["dtype"] == "f64"
    assert d["value"] > 0 and d["value"] == d["cpu_baseline"]["value"]
    # the line's time is the time the timed steps took: value and ms_per_step agree
    assert abs(d["value"] * d["ms_per_step"] / 1e3 / 17 ** 3 - 1) < 1e-9
    assert d["ms_per_step"] * d["steps"] / 1e3 <= d["wall_s"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert "workload" in d["config"]
