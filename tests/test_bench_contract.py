"""bench.py's reference arm runs on the host cores only: its one JSON line keeps the
contract's keys (the device arm is covered by the GPU run of bench.py itself)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "random_triangles",
                        "--steps", "2", "--warmup", "3", "--cpu-seconds", "2"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    j = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in j, key
    assert j["impl"] == "reference" and j["value"] > 0 and j["steps"] >= 1
    assert j["warmup"] == 3  # the requested warm-up frames ran
    assert j["higher_is_better"] is True and j["config"]["workload"]
    assert j["cpu_baseline"]["kind"] == "port" and j["cpu_baseline"]["cores"] >= 1
    assert j["e2e"]["h2d_bytes_per_step"] == 0 and j["e2e"]["d2h_bytes_per_step"] == 0
    assert abs(j["ms_per_step"] - 1e3 / j["value"]) < 0.01 * j["ms_per_step"] + 0.01


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "random_triangles",
                        "--steps", "1", "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600, check=True)
    assert not [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
