"""The benchmark's reference arm, run on the host cores as its launcher runs it.

`bench.py --impl reference` times the reference algorithm (the oracle, a
restatement of the reference's scalar code) on the whole headline workload
(the full matrix, three formats). Its JSON line must carry the same metric, unit, direction
and workload as the GPU arm's line, so that the two can be compared, plus a
`cpu_baseline` and an `e2e` with no host-device bytes. Under torchrun only
rank 0 runs it; the other ranks exit 0 and print nothing.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                           "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=300)


def test_reference_line_matches_gpu_arm_contract():
    pytest.importorskip("oracle.oracle")
    import bench
    r = _run({})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC
    assert line["unit"] == "GB/s" and line["higher_is_better"] is True
    assert line["config"] == {"workload": bench.WORKLOAD}   # the same work, no sample
    assert line["value"] > 0 and line["steps"] == 1
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["unit"] == "GB/s"
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == "GB/s"
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
