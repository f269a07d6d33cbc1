"""bench.py's reference arm on the CPU: the JSON line it prints for an LU-MZ
and an SP-MZ workload carries the contract's keys (the oracle port timed on
the host cores, no host-device traffic)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("workload", ["lu-a", "sp-a"])
def test_reference_arm_prints_the_contract_line(workload):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", workload,
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "Mgridpt-steps/s" and line["unit"] == "Mgridpt-steps/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 3
    assert line["dtype"] == "f64" and line["data"] == "synthetic"
    assert isinstance(line["config"]["workload"], str) and line["config"]["points"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["sample"].split(" after")[0] in ("1 SSOR iteration", "1 full time step"), cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
