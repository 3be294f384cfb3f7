"""bench.py's reference arm on the CPU: one JSON line with the measurement contract's keys.

The reference arm times the oracle's restatement of the path (the reference's Fortran build
is unavailable) on the host cores, on the GPU arm's workload, metric and unit; its `e2e` moves
no bytes between host and device."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["metric"].startswith("Mcell-steps/s at 1024^2") and d["unit"] == "Mcell-steps/s"
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["value"] > 0
    # the GPU arm's config, key for key: both arms report the same workload
    assert set(d["config"]) == {"workload", "nx", "ny", "ns", "parallelism", "l2"}
    assert d["config"]["nx"] == 1024 and d["config"]["ns"] == 256
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
