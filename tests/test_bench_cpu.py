"""bench.py's reference arm on the CPU: the timed CPU implementation of the
pair loops (the oracle port, one process per host core) prints one JSON
line with the fields the benchmark's consumers read, and under a
multi-process launch only rank 0 works and prints.
"""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, env_extra=None, timeout=300):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(REPO, "bench.py")] + args, cwd=REPO,
                          env=env, capture_output=True, text=True, timeout=timeout)


@pytest.mark.slow
def test_reference_arm_prints_one_line_with_the_contract_fields():
    proc = _run(["--impl", "reference", "--workload", "small", "--steps", "10",
                 "--warmup", "3"])
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [l for l in proc.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "pairs/s" and d["higher_is_better"] is True
    assert d["steps"] == 10 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == "small"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["per_core_value"] > 0 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_without_work():
    proc = _run(["--impl", "reference", "--workload", "small", "--steps", "10",
                 "--warmup", "3"], env_extra={"RANK": "1", "WORLD_SIZE": "2"}, timeout=120)
    assert proc.returncode == 0, proc.stderr[-2000:]
    assert proc.stdout.strip() == ""
