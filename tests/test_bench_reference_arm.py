"""The bench's reference arm on the host cores (no GPU): the JSON line it
prints for a small workload, and the silent exit of a rank other than 0."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(extra_env, *args):
    env = dict(os.environ, **extra_env)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                          capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)


def test_reference_arm_line_on_a_small_workload():
    r = _bench({"OMP_NUM_THREADS": "2"}, "--workload", "dambreak_small", "--steps", "3", "--warmup", "2")
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] and line["unit"] == "particle-steps/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["steps"] == 1 and line["steps_requested"] == 3 and line["warmup"] == 2
    assert line["config"]["workload"].startswith("dambreak_small")
    assert line["config"]["fluid_particles"] == 1250
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["sample"].startswith("dambreak_small itself (1250 fluid")
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _bench({"RANK": "1", "WORLD_SIZE": "2"}, "--workload", "dambreak_small", "--steps", "1",
               "--warmup", "0")
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
