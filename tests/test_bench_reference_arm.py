"""bench.py's reference arm runs on the host alone (the CPU oracle, never the
GPU library): a bounded sample of the 1D workload prints the benchmark line
with impl "reference"; the default 2^20-point workload, which the oracle
cannot assemble in bounded time, prints its unavailable line and exits 0."""
import json
import os
import subprocess
import sys

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _run(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"] + list(args),
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_on_a_cpu_workload():
    d = _run("--workload", "1d_rbf_32768", "--steps", "1", "--warmup", "0", "--rhs", "1")
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "solves/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["rel_err_vs_xtrue"] < 1e-6


def test_reference_arm_of_the_default_workload_is_unavailable():
    d = _run()
    assert d["impl"] == "reference" and "unavailable" in d
