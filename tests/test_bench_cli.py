"""bench.py's reference arm on a tiny workload (CPU only: the arm times the
reference's numpy simulator, no GPU is involved)."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_its_json_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--n", "10", "--depth", "2", "--steps", "1", "--warmup", "0"]
    env = {k: v for k, v in os.environ.items() if k not in ("PYTHONPATH", "CIRQ_GB300_CIRQ_PATH")}
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd="/", env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "gate-updates/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "reference"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert "10q" in line["config"]["workload"]


def test_reference_arm_other_ranks_exit_quietly():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "10",
           "--depth", "2", "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd="/", env=env)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
