"""The N-GPU bench path on the CPU: world_size-2 gloo ranks.

The ADI step does not shard across GPUs here (replicas only): each rank runs
the whole workload on its own GPU, and the job's figure takes the slowest
rank's time with the points of all ranks.  These tests run that host logic
(bench.whole_job) over a real gloo process group, and check that the
reference arm's non-zero ranks exit without work.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
rank = int(os.environ["RANK"]); world = int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo")
ms_local = [4.0, 5.0][rank]
ms_max, value = bench.whole_job(ms_local, pts=1000, steps=10, world=world, dist=dist, device="cpu")
dist.barrier()
dist.destroy_process_group()
print(json.dumps({{"rank": rank, "ms_max": ms_max, "value": value}}))
"""


def _spawn(world, port, script, extra_env=None):
    procs = []
    for rank in range(world):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", script], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for pr in procs:
        out, err = pr.communicate(timeout=120)
        assert pr.returncode == 0, err
        outs.append(out)
    return outs


def test_whole_job_takes_the_slowest_rank_and_all_ranks_points():
    outs = _spawn(2, 29561, RANK_SCRIPT.format(root=str(ROOT)))
    res = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    for r in res:
        assert r["ms_max"] == 5.0
        assert r["value"] == pytest.approx(1000 * 2 * 10 / 5e-3 / 1e6)


def test_reference_arm_other_ranks_exit_without_work():
    script = ("import sys; sys.path.insert(0, {root!r}); import bench; "
              "sys.argv = ['bench.py', '--impl', 'reference', '--gpus', '2']; sys.exit(bench.main())").format(root=str(ROOT))
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
