"""bench.py's reference arm on the CPU: one JSON line with the contract's
keys, on small workloads (the arm times the oracle on the host cores)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("workload,extra", [("swe", ["--n", "20"]), ("poisson", ["--n", "40"]),
                                            ("poisson-fv", ["--n", "20"]),
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


@pytest.mark.parametrize("workload,extra", [("swe", ["--n", "16"]), ("poisson", ["--n", "24"]),
                                            ("poisson-fv", ["--n", "16"]),
                                            ("batched", ["--count", "3", "--nmin", "8", "--nmax", "12"])])
def test_reference_arm_uses_no_native_code_and_our_config(workload, extra):
    """The reference arm builds its inputs with the oracle alone (this
    package's native library is never loaded) and prints the config dict
    our arm prints for the same arguments."""
    code = (
        "import sys, json, io, contextlib\n"
        f"sys.path.insert(0, {str(ROOT)!r})\n"
        "import bench\n"
        f"sys.argv = ['bench.py', '--impl', 'reference', '--workload', {workload!r}, '--steps', '1', "
        f"'--warmup', '0', *{extra!r}]\n"
        "buf = io.StringIO()\n"
        "with contextlib.redirect_stdout(buf):\n"
        "    bench.main()\n"
        "from easier_gb300 import _lib\n"
        "print(json.dumps({'line': json.loads(buf.getvalue().strip().splitlines()[-1]), "
        "'native_loaded': _lib._LIB is not None}))\n")
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    out = json.loads(res.stdout.strip().splitlines()[-1])
    assert out["native_loaded"] is False
    sys.path.insert(0, str(ROOT))
    import argparse
    import bench
    a = argparse.Namespace(workload=workload, n=None, dt=None, dtype="f32", precision=None, count=256, nmin=32,
                           nmax=512, seed=None)
    for k, v in zip(extra[::2], extra[1::2]):
        setattr(a, k.lstrip("-"), int(v))
    if a.n is None:
        a.n = 2000 if workload == "swe" else 1000
    a.dt = 5e-4 if a.n <= 1000 else 2.5e-4
    a.precision = "fast" if workload == "swe" else "native"
    a.seed = 1 if workload == "gnn" else 0
    want = {"swe": bench.swe_config, "poisson": bench.poisson_config, "poisson-fv": bench.poisson_config,
            "batched": bench.batched_config}[workload](a, 1)
    assert out["line"]["config"] == want
