"""bench.py's reference arm on the CPU: one JSON line with the contract's
keys, on small workloads (the arm times the oracle on the host cores)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("workload,extra", [("swe", ["--n", "20"]), ("poisson", ["--n", "40"]),
                                            ("batched", ["--count", "3", "--nmin", "8", "--nmax", "12"])])
def test_reference_arm_json_line(workload, extra):
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", workload,
           "--steps", "2", "--warmup", "1", *extra]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    for key in ("metric", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "config", "dtype"):
        assert key in line, key
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
