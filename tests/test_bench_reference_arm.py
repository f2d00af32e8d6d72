"""The bench's reference arm (`bench.py --impl reference`) on the host cores: it
prints one JSON line with the headline's metric, unit and workload, marked
"impl": "reference", with its CPU baseline described and an end-to-end entry
of zero copied bytes.  Runs without a GPU (a short sample per step)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup",
                        "1", "--ref-seconds", "1.0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    if "unavailable" in line:  # the reference could not be built on this machine: the line says why
        assert line["impl"] == "reference" and line["unavailable"]
        return
    assert line["impl"] == "reference"
    assert line["metric"].startswith("EM samples/s") and line["unit"] == "Msample-iter/s"
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert abs(cb["value"] - line["value"]) <= 1e-9 * max(1.0, line["value"])
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "4096 regions" in line["config"]["workload"]
