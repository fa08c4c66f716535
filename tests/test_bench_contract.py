"""bench.py's output contract, checked on the CPU: the reference arm (the oracle on the host cores)
prints one JSON line with the keys and meanings the line must carry."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_line(oracle_mod):
    d = _run("--impl", "reference", "--workload", "dam_break_27k", "--steps", "2", "--warmup", "1")
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["metric"] == "27k-particle PBF steps/s" and d["unit"] == "steps/s"
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["higher_is_better"] is True and d["value"] > 0
    assert abs(d["ms_per_step"] - 1000.0 / d["value"]) < 1e-6 * d["ms_per_step"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"] and cb["unit"] == "steps/s"
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == "steps/s"
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"] == "dam_break_27k"


def test_batched_reference_arm_is_unavailable():
    d = _run("--impl", "reference", "--workload", "batched_256", "--steps", "1", "--warmup", "1")
    assert d["impl"] == "reference" and "unavailable" in d
