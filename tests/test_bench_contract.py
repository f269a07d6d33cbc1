"""bench.py's reference arm on the CPU: the JSON line it prints for an LU-MZ
and an SP-MZ workload carries the contract's keys (the oracle port timed on
the host cores, no host-device traffic), its `config` has the GPU arm's keys
and values apart from `variant`, and the process maps no product library."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("workload", ["lu-a", "sp-a"])
def test_reference_arm_prints_the_contract_line(workload):
    # run the arm in-process and report which shared objects it mapped
    prog = ("import runpy, sys\n"
            f"sys.argv = ['bench.py', '--impl', 'reference', '--workload', '{workload}', '--steps', '1', "
            "'--warmup', '3']\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\nexcept SystemExit as e:\n"
            "    assert not e.code, e.code\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('MAPPED_PRODUCT', 'libnpbmz_gpu' in maps)\n")
    r = subprocess.run([sys.executable, "-c", prog], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.strip().splitlines()
    assert out[-1] == "MAPPED_PRODUCT False", out[-1]
    line = json.loads(out[-2])
    assert line["impl"] == "reference"
    assert line["metric"] == "Mgridpt-steps/s" and line["unit"] == "Mgridpt-steps/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 3
    assert line["dtype"] == "f64" and line["data"] == "synthetic"
    cfg = line["config"]
    assert isinstance(cfg["workload"], str) and cfg["points_per_gpu"] > 0
    sys.path.insert(0, str(ROOT))
    import bench

    kind, cls, desc = bench.WORKLOADS[workload]
    if kind == "LU":
        gpu_cfg = bench.workload_config(desc, cfg["points_per_gpu"], cfg["zones"], 1, "x")
    else:
        gpu_cfg = bench.workload_config(desc, cfg["points_per_gpu"], cfg["zones"], 1, "x", bench.SEED,
                                        {1: 0, 2: 1, 4: 2, 8: 3}[cfg["energy_row_scale"]])
    assert {k: v for k, v in cfg.items() if k != "variant"} == {k: v for k, v in gpu_cfg.items() if k != "variant"}
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["sample"].split(" after")[0] in ("1 SSOR iteration", "1 full time step"), cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
