"""bench.py's reference arm on the CPU: the JSON line it prints (one line, the
same metric and config keys as the GPU arm, a cpu_baseline describing the run,
an e2e object with no copies), and under torchrun only rank 0 runs and prints."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(env_extra, *args):
    env = dict(os.environ)
    env.update(env_extra)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                       capture_output=True, text=True, env=env, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_prints_one_contract_line():
    lines = _bench({"RANK": "0", "WORLD_SIZE": "1"}, "--n", "1500", "--steps", "2", "--warmup", "3",
                   "--ref-budget", "30")
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "points/s" and d["higher_is_better"] is True
    for key in ("metric", "value", "n_gpus", "steps", "warmup", "ms_per_step", "scaling", "vs_baseline", "dtype",
                "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["steps"] >= 1
    assert abs(d["value"] - 1500 / (d["ms_per_step"] / 1000.0)) < 1e-6 * d["value"]
    assert d["config"]["workload"] and d["config"]["n"] == 1500
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_without_work():
    assert _bench({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--n", "1500", "--steps", "1") == []
