"""Benchmark: GMRES time-to-1e-10 and matvec HBM GB/s of the GB300 H2*
operator, mixed precision (FP32 inner GMRES + FP64 iterative refinement)
against the plain FP64 GPU form, with the CPU oracle timed beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

A step is one solve of A x = b to relative residual 1e-10 from x0 = 1, b =
A_dense x_true (manufactured solution, FP64 dense product on the GPU), with
the compressed operator resident in HBM. value = solves per second of the
mixed form over all ranks. Multi-GPU runs are independent replicas (one
problem per GPU, no collective on the data path).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GMRES time-to-1e-10 & matvec HBM GB/s: mixed+batched+learned vs plain FP64 GPU"

WORKLOADS = {
    # configs[1]: 2D H2* integral equation, 256^2 grid, nmax 64, NCA tol 1e-10
    "2d_ie_65536": dict(dim=2, form=0, choice=0, tol=10, grid=256, leaf=8, gtol=10,
                        desc="2D H2* IE (choice 0), N=65536 (256^2 grid on [-1,1]^2), nmax=64, NCA tol 1e-10, "
                             "GMRES to 1e-10"),
    # configs[0]: 1D H2* (HSS) RBF, N=32768, nmax 64
    "1d_rbf_32768": dict(dim=1, form=0, choice=1, tol=10, grid=32768, leaf=64, gtol=10,
                         desc="1D H2* RBF (choice 1), N=32768 grid on [-1,1], nmax=64, NCA tol 1e-10, GMRES to 1e-10"),
}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples at 100 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), line.strip()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        rows = [s for (t, s) in self.samples if t0 <= t <= t1] or [s for (_, s) in self.samples]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            f = [x.strip() for x in r.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_problem(wl, device):
    import h2weak_gb300 as hw
    from h2weak_gb300 import synth
    dim = wl["dim"]
    nlev = hw.levels_for(dim, wl["grid"], wl["leaf"])
    N = wl["grid"] ** dim
    op = hw.H2Operator(dim, wl["form"], wl["choice"], wl["tol"], nlev, kernel_n=N,
                       diag_n=2 * N if dim == 1 else N, device=device)
    op.gen_grid(wl["grid"])
    op.build_tree()
    xt = synth.normal(synth.config_seed(1, 0), N)
    return op, nlev, xt


def cpu_oracle_solves(wl, steps, warmup):
    """The CPU oracle (restatement of the reference's algorithm) on the host
    cores: assembly, then `warmup` + `steps` FP64 GMRES solves."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import h2weak_gb300 as hw
    from h2weak_gb300 import synth
    from oracle import Oracle
    dim = wl["dim"]
    nlev = hw.levels_for(dim, wl["grid"], wl["leaf"])
    hop = hw.H2Operator(dim, wl["form"], wl["choice"], wl["tol"], nlev, device=-1)
    hop.gen_grid(wl["grid"])
    pts = hop.points()
    N = len(pts)
    t0 = time.time()
    o = Oracle(dim, wl["form"], pts, nlev, wl["tol"], wl["choice"], N, 2 * N if dim == 1 else N)
    t_asm = time.time() - t0
    xt = synth.normal(synth.config_seed(1, 0), N)
    # right-hand side from the compressed operator (the dense O(N^2) product is
    # the GPU's job; the timed quantity here is the solve)
    b = o.matvec(xt)
    for _ in range(warmup):
        o.gmres(b, max_iter=500, tol_pow=wl["gtol"])
    t0 = time.time()
    its = []
    for _ in range(steps):
        _, it, res = o.gmres(b, max_iter=500, tol_pow=wl["gtol"])
        its.append(it)
    t = time.time() - t0
    t0 = time.time()
    nmv = 5
    for _ in range(nmv):
        o.matvec(xt)
    t_mv = (time.time() - t0) / nmv
    return dict(t_solve=t / steps, iters=its[-1], t_asm=t_asm, t_mv=t_mv, mem=o.memory(), N=N,
                cores=int(os.environ.get("OMP_NUM_THREADS", os.cpu_count())))


def run_reference(args, wl):
    steps = max(1, args.steps)
    r = cpu_oracle_solves(wl, steps, max(0, min(args.warmup, 1)))
    v = 1.0 / r["t_solve"]
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": r["t_solve"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": wl["desc"], "N": r["N"], "form": "H2*", "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": r["cores"], "kind": "port",
                             "sample": "%d full FP64 GMRES solves to 1e-10 of the workload on the host cores "
                                       "(CPU oracle restating the reference's algorithm; assembly %.2fs untimed)"
                                       % (steps, r["t_asm"])},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gmres_iters": r["iters"], "matvec_ms": r["t_mv"] * 1e3,
            "matvec_gbs": 8.0 * r["mem"] / r["t_mv"] / 1e9}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="2d_ie_65536", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, wl)
        return

    import torch
    import torch.distributed as dist
    import h2weak_gb300 as hw
    torch.cuda.set_device(local)
    if world > 1:
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", rank=rank, world_size=world, device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    hw.build()
    op, nlev, xt = make_problem(wl, local)
    N = op.N
    torch.cuda.synchronize()
    t0 = time.time()
    op.assemble(hw.ASSEMBLE_NCA)
    t_asm = time.time() - t0
    storage = op.storage_entries()
    dev = torch.device("cuda", local)
    xt_d = torch.from_numpy(xt).to(dev)
    b_d = torch.empty(N, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    hw.lib().h2w_dense_matvec(op.h, xt_d.data_ptr(), b_d.data_ptr(), 0, N, hw.DEVICE)
    ones_d = torch.ones(N, dtype=torch.float64, device=dev)
    x_d = torch.empty_like(ones_d)

    def solve_mixed():
        x_d.copy_(ones_d)
        torch.cuda.synchronize()
        return op.gmres_ir_device(b_d.data_ptr(), x_d.data_ptr(), max_outer=20, inner_iter=200,
                                  tol_pow=wl["gtol"])

    def solve_fp64():
        x_d.copy_(ones_d)
        torch.cuda.synchronize()
        return op.gmres_device(b_d.data_ptr(), x_d.data_ptr(), max_iter=500, tol_pow=wl["gtol"])

    def timed(fn, k):
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = hw.launch_count()
        t0w = time.time()
        e0.record()
        out = None
        for _ in range(k):
            out = fn()
        e1.record()
        torch.cuda.synchronize()
        t1w = time.time()
        barrier()
        ms = e0.elapsed_time(e1)
        if world > 1:
            tt = torch.tensor([ms], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            ms = float(tt.item())
        return ms, out, hw.launch_count() - l0, (t0w, t1w)

    K, W = max(1, args.steps), max(3, args.warmup)
    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(W):
        solve_mixed()
    ms_mixed, out_mixed, launches, win = timed(solve_mixed, K)
    clocks.stop()
    outer, inner, res_mixed = out_mixed
    err_mixed = float(torch.linalg.norm(x_d - xt_d) / torch.linalg.norm(xt_d))

    for _ in range(W):
        solve_fp64()
    ms_fp64, out_fp64, _, _ = timed(solve_fp64, K)
    it64, res64 = out_fp64
    err_fp64 = float(torch.linalg.norm(x_d - xt_d) / torch.linalg.norm(xt_d))

    # end to end through the C ABI with pinned host buffers (b and x0 in, x out)
    b_h = b_d.cpu().pin_memory()
    x_h = torch.ones(N, dtype=torch.float64).pin_memory()

    def solve_e2e():
        x_h.fill_(1.0)
        return op.gmres_ir_device(b_h.data_ptr(), x_h.data_ptr(), max_outer=20, inner_iter=200,
                                  tol_pow=wl["gtol"], where=hw.HOST)

    for _ in range(W):
        solve_e2e()
    ms_e2e, _, _, _ = timed(solve_e2e, K)

    # roofline: profiled repeat of the timed mixed steps; per phase of the
    # block-row GEMV, algorithmic bytes per launch / mean launch time
    op.profile(True)
    for _ in range(K):
        solve_mixed()
    torch.cuda.synchronize()
    prof = {}
    for prec, nm in ((hw.PREC_FP32, "fp32"), (hw.PREC_FP64, "fp64")):
        la, ms, by = op.profile_phases(prec)
        prof[nm] = (la, ms, by)
    op.profile(False)
    # isolated matvecs per precision: per-phase device time
    phase_us = {}
    y_d = torch.empty_like(x_d)
    for prec, nm in ((hw.PREC_FP32, "fp32"), (hw.PREC_FP64, "fp64")):
        for _ in range(3):
            op.matvec_device(xt_d.data_ptr(), y_d.data_ptr(), precision=prec)
        op.profile(True)
        for _ in range(20):
            op.matvec_device(xt_d.data_ptr(), y_d.data_ptr(), precision=prec)
        torch.cuda.synchronize()
        la, ms, by = op.profile_phases(prec)
        op.profile(False)
        phase_us[nm] = {"us": [round(float(m) / max(int(l), 1) * 1e3, 2) for m, l in zip(ms, la)],
                        "MB": [round(float(b) / 1e6, 2) for b in by],
                        "total_us": round(float(ms.sum()) / 20 * 1e3, 1)}
    peak, peak_kind = load_peaks()
    # entries 0..P-1: per-phase launches (phased mode); entry P: whole-matvec
    # cooperative launches (default mode)
    best = None
    for nm, (la, ms, by) in prof.items():
        for q in range(len(la)):
            if la[q] == 0:
                continue
            if best is None or ms[q] > best[2]:
                best = (nm, q, float(ms[q]), int(la[q]), float(by[q]))
    nm, q, msq, laq, byq = best
    whole = q == len(prof[nm][0]) - 1
    tot_ms = sum(float(p[1].sum()) for p in prof.values())
    achieved = byq / (msq / laq / 1e3) / 1e9
    ctype = "float" if nm == "fp32" else "double"

    def per_mv(p):
        la, ms, by = p
        n = int(la.max()) if la.size else 0
        if n == 0:
            return 0.0, 0.0
        t = float(ms.sum()) / n
        b = float(by[-1]) if la[-1] else float((by * (la > 0)).sum())
        return t, b / (t / 1e3) / 1e9
    mv32_ms, mv32_gbs = per_mv(prof["fp32"])
    mv64_ms, mv64_gbs = per_mv(prof["fp64"])
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None,
            "kernel": ("brg_coop_kernel<%s> (one cooperative launch = one whole matvec, %d phases)"
                       % (ctype, len(prof[nm][0]) - 1)) if whole else
                      ("brg_kernel<%s> phase %d of %d" % (ctype, q, len(prof[nm][0]) - 1)),
            "bytes_per_launch": byq, "launch_us": msq / laq * 1e3, "launches": laq,
            "share_of_gemv_time": msq / tot_ms if tot_ms else None,
            "peak_kind": (peak_kind + " (MEASURED_PEAKS.json hbm_gbs)") if peak_kind == "measured" else peak_kind}

    # CPU baseline: the oracle on this host's cores
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        r = cpu_oracle_solves(wl, 1, 0)
        cpu = {"value": 1.0 / r["t_solve"], "unit": "solves/s", "cores": r["cores"], "kind": "port",
               "sample": "1 full FP64 GMRES solve to 1e-10 of the same workload (CPU oracle, assembly %.2fs untimed, "
                         "%d iterations, matvec %.1f ms)" % (r["t_asm"], r["iters"], r["t_mv"] * 1e3)}

    value = K * world / (ms_mixed / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms_mixed / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": wl["desc"], "N": N, "nlevels": nlev, "form": "H2*",
                   "solver": "FP32-operator inner GMRES (FP64 Arnoldi) + FP64 iterative refinement",
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "no flush: FP64 operator %.0f MB, FP32 %.0f MB, both > 129 MB L2" %
                         (op.operator_bytes(hw.PREC_FP64) / 1e6, op.operator_bytes(hw.PREC_FP32) / 1e6)},
        "e2e": {"value": K * world / (ms_e2e / 1e3), "unit": "solves/s", "h2d_bytes_per_step": 16 * N,
                "d2h_bytes_per_step": 8 * N},
        "gpu_launches": int(launches),
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(*win),
        "mixed": {"ms_per_solve": ms_mixed / K, "outer": outer, "inner_total": inner, "resid": res_mixed,
                  "rel_err_vs_xtrue": err_mixed, "fp32_matvec_ms": mv32_ms, "fp32_matvec_gbs": mv32_gbs},
        "fp64": {"ms_per_solve": ms_fp64 / K, "iters": it64, "resid": res64, "rel_err_vs_xtrue": err_fp64,
                 "matvec_ms": mv64_ms, "matvec_gbs": mv64_gbs, "speedup_mixed_over_fp64": ms_fp64 / ms_mixed},
        "assembly_s": t_asm, "storage_entries": storage, "phases": phase_us,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
