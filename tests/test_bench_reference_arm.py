"""bench.py --impl reference runs without a GPU (the oracle's C restatement of
the Zig screen on the host cores) and prints one JSON line with the keys the
benchmark contract names."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    # the same metric, unit and direction as our arm's line
    sys.path.insert(0, ROOT)
    import bench

    assert (line["metric"], line["unit"], line["higher_is_better"]) == (bench.METRIC, "candidates/s", True)
    cfg = dict(line["config"])
    assert "candidates" in cfg.pop("sample")  # the timed prefix is named in the config
    assert cfg == bench.workload_config(bench.parse([]), 1)
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]


def test_reference_arm_config1():
    """--workload config1 on the reference arm: the first configuration's model,
    lambda and keep."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "config1", "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["config"]["lambda"] == 1_000_000 and line["config"]["keep"] == 32
    assert "153" in line["config"]["surrogate"] and line["value"] > 0
