"""bench.py's reference arm runs on the host alone (the CPU oracle, never the
GPU library): a bounded sample of the 1D workload prints the benchmark line
with impl "reference"; the default 2^20-point workload, which the oracle
cannot assemble in bounded time, times FP64 solves of the first 2^15 points
of the same stream and scales them to one full solve."""
import json
import os
import subprocess
import sys

import numpy as np

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


def test_reference_arm_of_the_default_workload_scales_a_sample():
    d = _run("--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference" and d["unit"] == "solves/s" and d["higher_is_better"]
    s = d["sample"]
    assert s["N"] == 32768 and s["nlevels"] == 3 and s["rel_err_vs_xtrue"] < 1e-9
    # one full solve = the sample's solve x (E x (iterations + 1)) over the sample's
    scale = 48360650568 * 29 / (s["storage_entries"] * (s["gmres_iters"] + 1))
    assert abs(s["scale_to_full_solve"] / scale - 1) < 1e-12
    assert abs(d["ms_per_step"] / (s["ms_per_solve"] * scale) - 1) < 1e-9
    assert abs(d["value"] * d["ms_per_step"] / 1e3 - 1) < 1e-9
    assert d["cpu_baseline"]["value"] == d["value"] and d["config"]["N"] == 1048576


def test_cpu_sample_is_a_prefix_of_the_workload():
    """The sample's points and x_true are the first n of the workload's own
    streams; its tree depth follows the same rule (at most nmax points per
    leaf on average)."""
    sys.path.insert(0, ROOT)
    import bench
    wl = bench.WORKLOADS["3d_rbf_1048576"]
    syn = bench.load_synth()
    full = syn.uniform_points(syn.config_seed(5), 1 << 17, 3)
    assert np.array_equal(syn.uniform_points(syn.config_seed(5), 4096, 3), full[:4096])
    assert np.array_equal(syn.normal(syn.config_seed(5, 1), 4096), syn.normal(syn.config_seed(5, 1), 1 << 17)[:4096])
    assert bench.random_levels(wl, 1 << 20) == 5 and bench.random_levels(wl, 32768) == 3
    r = bench.cpu_oracle_sample_random(wl, 1, 0, n_sample=4096)
    assert r["n"] == 4096 and r["nlev"] == 2 and r["err"] < 1e-9
    assert abs(r["t_full"] / (r["t_solve"] * r["scale"]) - 1) < 1e-12
