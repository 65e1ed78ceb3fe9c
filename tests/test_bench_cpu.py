"""bench.py's reference arm runs on the host alone: its JSON line carries the
keys the benchmark contract asks for (the same metric, unit and direction as
the GPU arm, the CPU baseline that produced it, an end-to-end entry with no
host-device bytes)."""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _last_json_line(text):
    lines = [ln for ln in text.splitlines() if ln.strip().startswith("{")]
    assert lines, text[-2000:]
    return json.loads(lines[-1])


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = _last_json_line(r.stdout)
    assert d["impl"] == "reference"
    if "unavailable" in d:  # the contract's fallback line
        assert isinstance(d["unavailable"], str) and d["unavailable"]
        return
    assert d["metric"] and d["unit"] == "atom·k/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0
    assert d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["unit"] == d["unit"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_bench_options():
    r = subprocess.run([sys.executable, "bench.py", "--help"], cwd=REPO, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0
    for opt in ("--gpus", "--steps", "--warmup", "--impl", "--only"):
        assert opt in r.stdout
