"""bench.py's JSON line for the reference arm (host cores only, so it runs
here): one line with the contract's keys, the reference marker and an e2e
object with no host-device bytes (CPU only)."""

import json
import os
import subprocess
import sys

ROOT = os.path.join(os.path.dirname(__file__), os.pardir)

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
        "cpu_baseline", "e2e", "impl"}


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "3000",
                        "--steps", "1", "--warmup", "0", "--cpu-sample-s", "0.5"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert KEYS <= set(d)
    assert d["impl"] == "reference" and d["unit"] == "cubes/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["config"]["workload"] == "disc4m_1024" and d["config"]["particles"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    # a bounded pixel sample scaled to a whole cube, flagged as such
    assert cb["extrapolated"] is True and 0 < cb["timed_fraction"] < 1
    assert d["e2e"] == {"value": d["value"], "unit": "cubes/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
