"""Benchmark: GMRES time-to-1e-10 and matvec HBM GB/s of the GB300 H2*
operator, mixed precision against the plain FP64 GPU form.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME] [--rhs R]

Default workload (3d_rbf_1048576): 3D H2* RBF on 2^20 uniform random points,
nmax 128, NCA tol 1e-10, the far-field M2L evaluated during each product. A
step is one solve of A x = b (b = A x_true, x0 = 1) to relative residual
1e-10 with the compressed operator resident in HBM: FP32-operator inner GMRES
and iterative refinement with FP64-accurate residuals. value = solves per
second over all ranks. Beside it: the plain FP64 GMRES solve of the same
system, assembly time, storage, the operator's error on exact dense rows.
The host cannot assemble this operator in bounded time (hours, 387 GB), so
the CPU oracle (cpu_baseline and --impl reference) times FP64 solves of a
bounded sample, the first 2^15 points of the same point stream, and scales
each to one full solve by the stored entries a solve streams.

Other workloads: 2d_ie_65536 (2D H2* integral equation, 256^2 grid): a step
solves A X = B for R = 64 right-hand sides together (one multi-vector product
per Arnoldi step), beside it batched FP64 GMRES and one right-hand side by
the single-vector mixed and plain FP64 solvers, and the CPU oracle timed on
the same workload (--impl reference). 1d_rbf_32768 likewise; 3d_rbf_131072 is
the default family at 2^17 points (for profiler captures).

Multi-GPU runs are independent replicas (one problem per GPU, no collective
on the data path).
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
    # 2D H2* integral equation, 256^2 grid, nmax 64, NCA tol 1e-10 (64 right-hand sides per step; the CPU
    # oracle runs beside it)
    "2d_ie_65536": dict(dim=2, form=0, choice=0, tol=10, grid=256, leaf=8, gtol=10,
                        desc="2D H2* IE (choice 0), N=65536 (256^2 grid on [-1,1]^2), nmax=64, NCA tol 1e-10, "
                             "GMRES to 1e-10"),
    # the default workload: 3D H2* RBF, 2^20 uniform random points, nmax 128, tol 1e-10; its stored
    # operator (about 4.8e10 entries) exceeds HBM, so the far-field M2L is evaluated during each product.
    # full_e / full_it: the full operator's stored-entry count (the reference's findMemory count, which
    # the assembly reports) and the plain FP64 GMRES iteration count on this system, both measured on a
    # GB300; they scale the CPU oracle's bounded sample to one full solve (cpu_oracle_sample_random)
    "3d_rbf_1048576": dict(dim=3, form=0, choice=1, tol=10, npts=1048576, nmax=128, gtol=10, single=True,
                           full_e=48360650568, full_it=28,
                           desc="3D H2* RBF (choice 1), N=1048576 uniform random points in [-1,1)^3 "
                                "(splitmix64 stream), nmax=128 (5 levels), NCA tol 1e-10, GMRES to 1e-10, "
                                "one right-hand side per solve; far-field M2L evaluated during each product"),
    # the same family at 2^17 points (4 levels): a case small enough for ncu captures of the far-field kernel
    "3d_rbf_131072": dict(dim=3, form=0, choice=1, tol=10, npts=131072, nmax=128, gtol=10, single=True,
                          full_e=3966023186, full_it=21,
                          desc="3D H2* RBF (choice 1), N=131072 uniform random points in [-1,1)^3 "
                               "(splitmix64 stream), nmax=128 (4 levels), NCA tol 1e-10, GMRES to 1e-10, "
                               "one right-hand side per solve; far-field M2L evaluated during each product"),
    # the CPU-sized case: 1D H2* (HSS) RBF, N=32768, nmax 64
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


def max_over_ranks(v, world, device=None):
    """The slowest rank's figure: replicas end with their last rank, so a
    multi-GPU run's time is the maximum over ranks (torch.distributed, any
    backend; the value is the same on every rank)."""
    if world <= 1:
        return float(v)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, world, ms):
    """Whole-job throughput of independent replicas: every rank's units over
    the slowest rank's time (ms, the maximum over ranks)."""
    return units_per_rank * world / (ms / 1e3)


def nlevels_for(dim, n_param, leaf_param):
    """Tree depth as the reference's drivers compute it (1D/codes/main.cpp:13,
    2D/codes/main.cpp:13, 3D/codes/main.cpp:11)."""
    import math
    if dim == 1:
        return int(math.ceil(math.log(float(n_param) / leaf_param) / math.log(2)))
    if dim == 2:
        return int(math.ceil(2.0 * math.log(float(n_param) / leaf_param) / math.log(4)))
    return int(math.ceil(3 * math.log(float(n_param) / leaf_param) / math.log(8)))


def grid_points(dim, n):
    """The reference's uniform grid (set_Uniform_Nodes, 1D/codes/HODLR1Dtree.hpp:59-66,
    2D/codes/HODLR2Dtree.hpp:75-91, 3D/codes/HODLR3Dtree.hpp:82-102) with its
    point numbering, in numpy: node k = -1 + 2(k+1)/(n+1), the same operations
    in the same order as the library's h2w_gen_grid, so the points are bitwise
    the same. The CPU arm builds its points here and never loads the GPU library."""
    k = np.arange(n, dtype=np.float64)
    node = -1.0 + 2.0 * (k + 1.0) / (n + 1.0)
    if dim == 1:
        return node.reshape(n, 1)
    if dim == 2:
        j, kk = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        return np.stack([node[kk.ravel()], node[j.ravel()]], axis=1)
    j, kk, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return np.stack([node[kk.ravel()], node[j.ravel()], node[i.ravel()]], axis=1)


def load_synth():
    """The seeded generators (h2weak_gb300/synth.py, pure numpy) loaded by
    path, without importing the GPU package."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("h2w_synth", os.path.join(ROOT, "h2weak_gb300", "synth.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def common_config(wl, N, nlev, R):
    """The workload, identical in both arms' lines."""
    return {"workload": wl["desc"], "N": N, "nlevels": nlev, "form": "H2*", "rhs_per_step": R,
            "rhs": "columns N(0,1) from seeded splitmix64 streams, B = A X_true with the FP64 compressed "
                   "operator, X0 = 1", "tolerance": "relative residual 1e-%d per column" % wl["gtol"],
            "parallelism": "replicas (one problem per GPU)",
            "l2": "no flush: the compressed operator exceeds the 129 MB L2 (inputs larger than L2)"}


def make_problem(wl, device):
    import h2weak_gb300 as hw
    from h2weak_gb300 import synth
    dim = wl["dim"]
    nlev = nlevels_for(dim, wl["grid"], wl["leaf"])
    N = wl["grid"] ** dim
    op = hw.H2Operator(dim, wl["form"], wl["choice"], wl["tol"], nlev, kernel_n=N,
                       diag_n=2 * N if dim == 1 else N, device=device)
    op.gen_grid(wl["grid"])
    op.build_tree()
    xt = synth.normal(synth.config_seed(1, 0), N)
    return op, nlev, xt


def cpu_oracle_solves(wl, R, steps, warmup, budget_s=150.0):
    """The CPU oracle (the reference's algorithm restated in C++, OpenMP on
    every host core) on the same workload: assembly, then per step the FP64
    GMRES solves of the step's right-hand sides one after another (the
    reference solves one right-hand side per call). Every step solves all R
    columns when warmup + steps fit in budget_s, else the same number of
    columns from each step's sample (stated in the result)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    synth = load_synth()
    dim = wl["dim"]
    nlev = nlevels_for(dim, wl["grid"], wl["leaf"])
    pts = grid_points(dim, wl["grid"])
    N = len(pts)
    t0 = time.time()
    o = Oracle(dim, wl["form"], pts, nlev, wl["tol"], wl["choice"], N, 2 * N if dim == 1 else N)
    t_asm = time.time() - t0
    cols = [synth.normal(synth.config_seed(1, c), N) for c in range(R)]
    rhs = [o.matvec(x) for x in cols]
    t0 = time.time()
    _, it0, _ = o.gmres(rhs[0], max_iter=500, tol_pow=wl["gtol"])
    t_col = time.time() - t0
    per_step = max(1, min(R, int(budget_s / max(t_col * (steps + warmup), 1e-9))))
    for w in range(warmup):
        for c in range(per_step):
            o.gmres(rhs[(w * per_step + c) % R], max_iter=500, tol_pow=wl["gtol"])
    its, errs = [], []
    t0 = time.time()
    for k in range(steps):
        for c in range(per_step):
            q = (k * per_step + c) % R
            x, it, res = o.gmres(rhs[q], max_iter=500, tol_pow=wl["gtol"])
            its.append(it)
    t = time.time() - t0
    errs.append(float(np.linalg.norm(x - cols[q]) / np.linalg.norm(cols[q])))
    t0 = time.time()
    nmv = 10
    for _ in range(nmv):
        o.matvec(cols[0])
    t_mv = (time.time() - t0) / nmv
    return dict(t_step=t / steps, cols_per_step=per_step, t_solve=t / (steps * per_step), iters=max(its),
                t_asm=t_asm, t_mv=t_mv, mem=o.memory(), N=N, nlev=nlev, err=errs[-1],
                cores=int(os.environ.get("OMP_NUM_THREADS", os.cpu_count())))


def random_levels(wl, n):
    """Tree depth of a random-point workload: the fewest levels with at most
    nmax points per leaf on average."""
    import math
    return int(math.ceil(math.log(n / float(wl["nmax"])) / math.log(2.0 ** wl["dim"])))


def single_config(wl, N, nlev):
    """The random-point workload's config, identical in both arms' lines."""
    return {"workload": wl["desc"], "N": N, "nlevels": nlev, "form": "H2*", "rhs_per_step": 1,
            "rhs": "x_true N(0,1) from a seeded splitmix64 stream, b = A x_true with the FP64 compressed "
                   "operator, x0 = 1",
            "tolerance": "relative residual 1e-%d" % wl["gtol"], "parallelism": "replicas (one problem per GPU)",
            "l2": "no flush: the stored operator exceeds the 129 MB L2 (inputs larger than L2)"}


def cpu_oracle_sample_random(wl, steps, warmup, n_sample=32768):
    """The CPU oracle (the reference's algorithm restated in C++, OpenMP on
    every host core) on a bounded sample of a random-point workload whose full
    operator the host cannot assemble in bounded time (the 2^20-point one
    takes hours and 387 GB): the first n_sample points of the workload's own
    point stream, tree depth by the same rule, the same kernel and tolerances,
    x_true the first n_sample entries of the workload's, b = A x_true, x0 = 1.
    Assembly is untimed; each step is one FP64 GMRES solve of the sample,
    scaled to one solve of the full workload by the stored entries a solve
    streams, E x (iterations + 1): the full operator's E and FP64 iteration
    count are the workload's full_e / full_it. The products (the operator
    streamed once each) are about 96 % of the sample's solve; the rest, the
    Arnoldi work, grows as N x iterations^2 (77x to the full size, not 138x),
    so the scaled time is at most about 2 % high."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    synth = load_synth()
    n = min(n_sample, wl["npts"])
    nlev = random_levels(wl, n)
    pts = synth.uniform_points(synth.config_seed(5), n, wl["dim"])
    t0 = time.time()
    o = Oracle(wl["dim"], wl["form"], pts, nlev, wl["tol"], wl["choice"])
    t_asm = time.time() - t0
    xt = synth.normal(synth.config_seed(5, 1), n)
    b = o.matvec(xt)
    for _ in range(warmup):
        o.gmres(b, max_iter=500, tol_pow=wl["gtol"])
    ts = []
    for _ in range(steps):
        t0 = time.time()
        x, it, res = o.gmres(b, max_iter=500, tol_pow=wl["gtol"])
        ts.append(time.time() - t0)
    t0 = time.time()
    for _ in range(10):
        o.matvec(xt)
    t_mv = (time.time() - t0) / 10
    E = o.memory()
    scale = wl["full_e"] * (wl["full_it"] + 1.0) / (E * (it + 1.0))
    t_solve = sum(ts) / len(ts)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
    sample = ("one FP64 GMRES solve to 1e-%d per step of the first %d points of the workload's point stream (%d "
              "levels, E=%d stored entries, %d iterations, %.3f s; assembly %.1f s untimed) by the CPU oracle "
              "restating the reference's algorithm on %d host cores, scaled x%.1f to one solve of the full "
              "workload by stored entries streamed per solve, E x (iterations + 1) = %d x %d against %d x %d "
              "(the full E and FP64 iteration count measured on a GB300)"
              % (wl["gtol"], n, nlev, E, it, t_solve, t_asm, cores, scale, wl["full_e"], wl["full_it"] + 1, E,
                 it + 1))
    return dict(t_full=t_solve * scale, t_solve=t_solve, scale=scale, n=n, nlev=nlev, E=E, iters=it, res=res,
                err=float(np.linalg.norm(x - xt) / np.linalg.norm(xt)), t_asm=t_asm, t_mv=t_mv, cores=cores,
                sample=sample)


def run_single_random(args, wl, rank, world, local):
    """The 2^20-point 3D workload: one right-hand side per solve, b = A x_true with
    the FP64 compressed operator, x0 = 1. value = mixed-precision solves per
    second over all ranks (FP32 inner GMRES, FP64-accurate refinement); beside
    it the plain FP64 GMRES, the operator's error on exact dense rows, assembly
    time and storage. Multi-GPU runs are independent replicas (one problem per
    GPU, no collective on the data path)."""
    import torch
    import torch.distributed as dist
    import h2weak_gb300 as hw
    from h2weak_gb300 import synth
    torch.cuda.set_device(local)
    if world > 1:
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", rank=rank, world_size=world, device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    hw.build()
    N, dim = wl["npts"], wl["dim"]
    nlev = random_levels(wl, N)
    op = hw.H2Operator(dim, wl["form"], wl["choice"], wl["tol"], nlev, device=local)
    op.set_points(synth.uniform_points(synth.config_seed(5), N, dim))
    op.build_tree()
    op.set_option(hw.OPT_FAR_ON_THE_FLY, 1)
    # the mixed solver's accurate residuals: FP64-accurate double-FP32 far field on the FP32 pipes
    op.set_option(hw.OPT_IR_RESIDUAL, hw.PREC_DF64)
    torch.cuda.synchronize()
    t0 = time.time()
    op.assemble(hw.ASSEMBLE_NCA)
    torch.cuda.synchronize()
    t_asm = time.time() - t0
    dev = torch.device("cuda", local)
    # a stream of torch's own (not the legacy default stream) for the products, so
    # that CUDA events recorded on it bracket the library's launches
    strm = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(strm)
    st = strm.cuda_stream
    xt = torch.from_numpy(synth.normal(synth.config_seed(5, 1), N)).to(dev)
    b = torch.empty_like(xt)
    op.matvec_device(xt.data_ptr(), b.data_ptr(), precision=hw.PREC_FP64, stream=st)
    x = torch.empty_like(xt)
    gtol = wl["gtol"]

    def ev_time(fn, k):
        torch.cuda.synchronize()
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
        barrier()
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1), world, dev), out, hw.launch_count() - l0, (t0w, time.time())

    # products on this stream: FP32, double-FP32 and FP64, each with its far M2L kernel
    mv = {}
    y = torch.empty_like(xt)
    for prec, nm, reps in ((hw.PREC_FP32, "fp32", 5), (hw.PREC_DF64, "df64", 3), (hw.PREC_FP64, "fp64", 1)):
        op.matvec_device(xt.data_ptr(), y.data_ptr(), precision=prec, stream=st)
        ms, _, _, _ = ev_time(lambda: op.matvec_device(xt.data_ptr(), y.data_ptr(), precision=prec, stream=st), reps)
        mv[nm] = ms / reps

    def solve_mixed():
        x.fill_(1.0)
        return op.gmres_ir_device(b.data_ptr(), x.data_ptr(), max_outer=20, inner_iter=200, tol_pow=gtol)

    K, W = max(1, args.steps), max(3, args.warmup)
    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(W):
        solve_mixed()
    ms_m, out_m, launches, win = ev_time(solve_mixed, K)
    clocks.stop()
    outer, inner, res_m = out_m
    err_m = float(torch.linalg.norm(x - xt) / torch.linalg.norm(xt))
    # the far-field M2L kernel alone (CUDA events on this stream around each of its
    # launches), inside FP32 and double-FP32 products
    op.profile(True)
    for _ in range(5):
        op.matvec_device(xt.data_ptr(), y.data_ptr(), precision=hw.PREC_FP32, stream=st)
    op.matvec_device(xt.data_ptr(), y.data_ptr(), precision=hw.PREC_DF64, stream=st)
    fly32 = op.profile_fly(hw.PREC_FP32)
    flydf = op.profile_fly(hw.PREC_DF64)
    op.profile(False)
    # end to end: host b in, host x out through the C ABI
    b_h = b.cpu().pin_memory()
    x_h = torch.ones_like(b_h).pin_memory()

    def solve_e2e():
        x_h.fill_(1.0)
        return op.gmres_ir_device(b_h.data_ptr(), x_h.data_ptr(), max_outer=20, inner_iter=200, tol_pow=gtol,
                                  where=hw.HOST)

    ms_e2e, _, _, _ = ev_time(solve_e2e, 1)
    # plain FP64 GMRES, the comparison form (one timed solve)
    def solve_fp64():
        x.fill_(1.0)
        return op.gmres_device(b.data_ptr(), x.data_ptr(), max_iter=500, tol_pow=gtol)

    ms_64, out_64, _, _ = ev_time(solve_fp64, 1)
    it64, res64 = out_64
    err_64 = float(torch.linalg.norm(x - xt) / torch.linalg.norm(xt))
    dense_err = op.total_error(xt.cpu().numpy(), 1024)
    # the CPU baseline (one-GPU runs): the oracle on a bounded sample of this workload, after
    # every GPU timing so that the load on the host cores touches none of the GPU's figures
    cpu = {"value": None, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
           "sample": "timed on one-GPU runs only (--no-cpu-baseline skips it)"}
    if world == 1 and not args.no_cpu_baseline:
        try:
            r = cpu_oracle_sample_random(wl, 2, 0)
            cpu = {"value": 1.0 / r["t_full"], "unit": "solves/s", "cores": r["cores"], "kind": "port",
                   "sample": r["sample"]}
        except Exception as e:  # the GPU figures above still print
            cpu["sample"] = "CPU oracle failed: %s" % str(e)[:200]
    peak, peak_kind = load_peaks()
    stored = op.operator_bytes(hw.PREC_FP32)
    E = op.storage_entries()
    # Roofline. The unit is one FP32 product (the inner GMRES's matvec, 50 of them in a
    # solve): algorithmic bytes = 4 B x E (E the reference's storage count, every block
    # it stores, at the FP32 operator's width) + the FP64 input and output vectors, over
    # the product's CUDA-event time. The product streams its stored 30.8 GB and forms
    # the far-field M2L entries (84 % of E) from the points in m2l_fly32_sep_kernel,
    # which is bound by instruction issue, not DRAM (its own figures beside it).
    fl_n, fl_ms, fl_e = fly32
    fl_t = fl_ms / max(fl_n, 1)
    prod_bytes = 4.0 * E + 2 * 8.0 * N
    prod_gbs = prod_bytes / (mv["fp32"] * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": replica_throughput(K, world, ms_m), "unit": "solves/s", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": ms_m / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": single_config(wl, N, nlev),
        "solver": "mixed: FP32-operator inner GMRES + iterative refinement with FP64-accurate residuals (stored "
                  "passes FP64, far-field M2L in double-FP32 arithmetic), CUDA-graph Arnoldi loop; far-field M2L "
                  "evaluated from the points in every product; the plain form is FP64 throughout",
        "e2e": {"value": replica_throughput(1, world, ms_e2e), "unit": "solves/s", "h2d_bytes_per_step": 16 * N,
                "d2h_bytes_per_step": 8 * N},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "unit_of_work": "one FP32 product (stored passes + far-field M2L kernel)",
                     "achieved": prod_gbs, "peak": peak, "unit": "GB/s", "frac": prod_gbs / peak, "traffic": None,
                     "algorithmic_bytes": prod_bytes, "ms": mv["fp32"], "stored_fp32_bytes": stored,
                     "note": "achieved = (4 B x the reference's storage count E + 16 B x N) / the product's "
                             "CUDA-event time, against the measured HBM copy bandwidth (%s). The product reads "
                             "its stored %.1f GB and evaluates the far-field M2L entries (%.3g of E's %.3g) from "
                             "the points instead of reading them, so achieved can exceed the copy bandwidth; "
                             "stored_passes gives the HBM rate of the part that streams its operator. traffic "
                             "is null (three launches; DRAM bytes per far-field entry 0.062 in "
                             "profiles/m2l_fly32_sep_3d_rbf_131072.md)" % (peak_kind, stored / 1e9, fl_e, E),
                     "far_field_kernel": {"name": "m2l_fly32_sep_kernel", "bound": "instruction issue",
                                          "launch_ms": fl_t, "entries_per_launch": fl_e,
                                          "entries_per_s": fl_e / (fl_t * 1e-3) if fl_n else None,
                                          "share_of_product": fl_t / mv["fp32"] if fl_n else None},
                     # the part of the product that streams its operator from HBM: the stored
                     # passes (the product's time less the far-field kernel's), their FP32 bytes
                     "stored_passes": {"bytes": stored, "ms": mv["fp32"] - fl_t,
                                       "achieved_gbs": stored / ((mv["fp32"] - fl_t) * 1e-3) / 1e9
                                       if fl_n and mv["fp32"] > fl_t else None,
                                       "frac": stored / ((mv["fp32"] - fl_t) * 1e-3) / 1e9 / peak
                                       if fl_n and mv["fp32"] > fl_t else None}},
        "compute": {"flydf_ms": flydf[1] / max(flydf[0], 1), "flydf_entries_per_s":
                        flydf[2] / (flydf[1] / max(flydf[0], 1) * 1e-3) if flydf[0] else None},
        "cpu_baseline": cpu,
        "clocks": clocks.summary(*win),
        "mixed": {"ms_per_solve": ms_m / K, "outer": outer, "inner_total": inner, "resid": res_m,
                  "rel_err_vs_xtrue": err_m},
        "single_fp64": {"ms_per_solve": ms_64, "iters": it64, "resid": res64, "rel_err_vs_xtrue": err_64},
        "speedup_vs_plain_fp64": {"single_mixed_over_single_fp64": ms_64 / (ms_m / K)},
        "matvec_ms": mv, "operator_error_1024_dense_rows": dense_err,
        "assembly_s": t_asm, "storage_entries": E,
        "stored_bytes": {"fp64": op.operator_bytes(hw.PREC_FP64), "fp32": stored},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_reference(args, wl):
    steps = max(1, args.steps)
    R = max(1, min(64, args.rhs))
    r = cpu_oracle_solves(wl, R, steps, max(0, min(args.warmup, 1)))
    v = 1.0 / r["t_solve"]
    sample = ("%d of the step's %d right-hand sides per step (%s), each a full FP64 GMRES solve to 1e-%d on the "
              "host cores by the CPU oracle restating the reference's algorithm; assembly %.2fs untimed" %
              (r["cols_per_step"], R, "the whole step" if r["cols_per_step"] == R else "a bounded sample",
               wl["gtol"], r["t_asm"]))
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": r["t_solve"] * R * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": common_config(wl, r["N"], r["nlev"], R),
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": r["cores"], "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "solver": "unrestarted FP64 GMRES per right-hand side (iterative_solver::GMRES, "
                      "1D/codes/gmres.hpp:92-200), compressed operator matvec (OpenMP)",
            "gmres_iters": r["iters"], "rel_err_vs_xtrue": r["err"], "matvec_ms": r["t_mv"] * 1e3,
            "matvec_gbs": 8.0 * r["mem"] / r["t_mv"] / 1e9, "assembly_s": r["t_asm"], "storage_entries": r["mem"]}
    print(json.dumps(line), flush=True)


def run_reference_single(args, wl):
    """The reference arm of a random-point workload: per step one FP64 GMRES
    solve by the CPU oracle on the bounded sample, scaled to one full solve
    (cpu_oracle_sample_random); value = full solves per second."""
    steps = max(1, args.steps)
    r = cpu_oracle_sample_random(wl, steps, max(0, min(args.warmup, 1)))
    v = 1.0 / r["t_full"]
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": r["t_full"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": single_config(wl, wl["npts"], random_levels(wl, wl["npts"])),
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": r["cores"], "kind": "port",
                             "sample": r["sample"]},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "solver": "unrestarted FP64 GMRES (iterative_solver::GMRES, 3D/codes/gmres.hpp:92-200), compressed "
                      "matvec (OpenMP)",
            "sample": {"N": r["n"], "nlevels": r["nlev"], "storage_entries": r["E"], "gmres_iters": r["iters"],
                       "resid": r["res"], "rel_err_vs_xtrue": r["err"], "ms_per_solve": r["t_solve"] * 1e3,
                       "matvec_ms": r["t_mv"] * 1e3, "matvec_gbs": 8.0 * r["E"] / r["t_mv"] / 1e9,
                       "assembly_s": r["t_asm"], "scale_to_full_solve": r["scale"]}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="3d_rbf_1048576", choices=sorted(WORKLOADS))
    ap.add_argument("--rhs", type=int, default=64, help="right-hand sides solved together per step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            if wl.get("single"):
                run_reference_single(args, wl)
            else:
                run_reference(args, wl)
        return
    if wl.get("single"):
        run_single_random(args, wl, rank, world, local)
        return

    import torch
    import torch.distributed as dist
    import h2weak_gb300 as hw
    from h2weak_gb300 import synth
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
    R = max(1, min(64, args.rhs))
    torch.cuda.synchronize()
    t0 = time.time()
    op.assemble(hw.ASSEMBLE_NCA)
    t_asm = time.time() - t0
    storage = op.storage_entries()
    dev = torch.device("cuda", local)
    gtol = wl["gtol"]
    # single right-hand side: b = A_dense x_true (manufactured solution)
    xt_d = torch.from_numpy(xt).to(dev)
    b_d = torch.empty(N, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    hw.lib().h2w_dense_matvec(op.h, xt_d.data_ptr(), b_d.data_ptr(), 0, N, hw.DEVICE)
    torch.cuda.synchronize()
    x_d = torch.empty_like(b_d)
    # R right-hand sides: columns x_true_c (column 0 = x_true), B = A X_true with
    # the FP64 compressed operator (the dense O(N^2) product per column is left
    # to the sampled-row check below); column-major N x R = rows of an R x N tensor
    XT = np.stack([synth.normal(synth.config_seed(1, c), N) for c in range(R)], axis=0)
    XT_d = torch.from_numpy(XT).to(dev)
    B_d = torch.empty_like(XT_d)
    torch.cuda.synchronize()
    op.matvec_device(XT_d.data_ptr(), B_d.data_ptr(), nrhs=R, precision=hw.PREC_FP64)
    torch.cuda.synchronize()
    X_d = torch.empty_like(XT_d)
    op.set_option(hw.OPT_IR_RESIDUAL, hw.PREC_DF64)
    # target granularity picked by the autotuner on this operator and GPU
    # (multi-vector stream on the refinement step's product mix: four FP32
    # products per double-FP32 residual; single-vector stream on the FP32 product)
    tuned_xw, tuned_xw_ms = op.autotune(nrhs=R, precision=hw.TUNE_IR_MIX, reps=2)
    tuned_rs, tuned_rs_ms = op.autotune(nrhs=1, precision=hw.PREC_FP32, reps=5)

    def solve_batched():
        X_d.fill_(1.0)
        torch.cuda.synchronize()  # the library runs on its own stream
        return op.gmres_ir_batch_device(B_d.data_ptr(), X_d.data_ptr(), R, max_outer=20, inner_iter=200,
                                        tol_pow=gtol)

    def solve_batched_fp64():
        X_d.fill_(1.0)
        torch.cuda.synchronize()
        return op.gmres_batch_device(B_d.data_ptr(), X_d.data_ptr(), R, max_iter=400, tol_pow=gtol)

    def solve_mixed():
        x_d.fill_(1.0)
        torch.cuda.synchronize()
        return op.gmres_ir_device(b_d.data_ptr(), x_d.data_ptr(), max_outer=20, inner_iter=200, tol_pow=gtol)

    def solve_fp64():
        x_d.fill_(1.0)
        torch.cuda.synchronize()
        return op.gmres_device(b_d.data_ptr(), x_d.data_ptr(), max_iter=500, tol_pow=gtol)

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
        ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
        return ms, out, hw.launch_count() - l0, (t0w, t1w)

    def col_err(X):
        return float(torch.max(torch.linalg.norm(X - XT_d, dim=1) / torch.linalg.norm(XT_d, dim=1)))

    K, W = max(1, args.steps), max(3, args.warmup)
    # ---- the timed step: R right-hand sides, mixed precision, batched
    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(W):
        solve_batched()
    ms_b, out_b, launches, win = timed(solve_batched, K)
    clocks.stop()
    outer_b, inner_b, res_b = out_b
    err_b = col_err(X_d)
    # FP64 residual of the batched solution (host check) and the dense sampled rows
    Yb = torch.empty_like(X_d)
    op.matvec_device(X_d.data_ptr(), Yb.data_ptr(), nrhs=R, precision=hw.PREC_FP64)
    torch.cuda.synchronize()
    fp64_resid_b = float(torch.max(torch.linalg.norm(B_d - Yb, dim=1) / torch.linalg.norm(B_d, dim=1)))
    nrow = min(1024, N)
    yrows = torch.empty(nrow, dtype=torch.float64, device=dev)
    x0c = X_d[0].contiguous()
    hw.lib().h2w_dense_matvec(op.h, x0c.data_ptr(), yrows.data_ptr(), 0, nrow, hw.DEVICE)
    brows = torch.empty_like(yrows)
    xt0 = XT_d[0].contiguous()
    hw.lib().h2w_dense_matvec(op.h, xt0.data_ptr(), brows.data_ptr(), 0, nrow, hw.DEVICE)
    torch.cuda.synchronize()
    dense_rows_err = float(torch.linalg.norm(yrows - brows) / torch.linalg.norm(brows))
    # ---- beside it: batched FP64 GMRES, single-vector mixed and FP64 solves
    for _ in range(W):
        solve_batched_fp64()
    ms_b64, out_b64, _, _ = timed(solve_batched_fp64, K)
    it_b64 = int(np.max(out_b64[0]))
    err_b64 = col_err(X_d)
    for _ in range(W):
        solve_mixed()
    ms_mixed, out_mixed, _, _ = timed(solve_mixed, K)
    outer, inner, res_mixed = out_mixed
    err_mixed = float(torch.linalg.norm(x_d - xt_d) / torch.linalg.norm(xt_d))
    for _ in range(W):
        solve_fp64()
    ms_fp64, out_fp64, _, _ = timed(solve_fp64, K)
    it64, res64 = out_fp64
    err_fp64 = float(torch.linalg.norm(x_d - xt_d) / torch.linalg.norm(xt_d))

    # ---- end to end through the C ABI with pinned host buffers (B, X0 in; X out)
    B_h = B_d.cpu().pin_memory()
    X_h = torch.ones_like(B_h).pin_memory()

    def solve_e2e():
        X_h.fill_(1.0)
        return op.gmres_ir_batch_device(B_h.data_ptr(), X_h.data_ptr(), R, max_outer=20, inner_iter=200,
                                        tol_pow=gtol, where=hw.HOST)

    for _ in range(W):
        solve_e2e()
    ms_e2e, _, _, _ = timed(solve_e2e, K)

    # ---- roofline: profiled repeat of the timed steps (host-driven loop while
    # profiling), per precision of the multi-vector kernel
    peak, peak_kind = load_peaks()
    op.profile(True)
    for _ in range(K):
        solve_batched()
    torch.cuda.synchronize()
    kern = {}
    for prec, nm in ((hw.PREC_FP32, "fp32"), (hw.PREC_DF64, "df64"), (hw.PREC_FP64, "fp64")):
        la, ms, by = op.profile_multi(prec)
        if la:
            kern[nm] = dict(launches=la, ms=ms, bytes=by, us=ms / la * 1e3, gbs=by / (ms / la / 1e3) / 1e9)
    op.profile(False)
    tot = sum(k["ms"] for k in kern.values())
    top = max(kern, key=lambda k: kern[k]["ms"])
    tk = kern[top]
    ctype = {"fp32": "float, FP32", "df64": "double, double-FP32", "fp64": "double, FP64"}[top]
    rp = 16 if R <= 16 else (32 if R <= 32 else 64)
    # DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from the ncu captures of the
    # same launches on this workload: profiles/mw_flow_fp32_2d_ie_65536.md, mr_flow_df64_2d_ie_65536.md
    kname = (("mw_flow_kernel" if top == "fp32" and op.get_option(hw.OPT_PRODUCER_WARP) else "mr_flow_kernel")
             if op.get_option(hw.OPT_DATAFLOW) else "mr_coop_kernel")
    ncu_traffic = {("mw_flow_kernel", "fp32"): 361.970e6 + 72.415e6, ("mr_flow_kernel", "df64"): 896.444e6 + 188.591e6}
    # the multi-vector kernel multiplies every packed operator entry by R vectors: one FMA per
    # term (FP32), about twelve FP32 operations per term (double-FP32); nominal FP32 peak of
    # 152 SMs x 128 lanes x 2 flop x 2.07 GHz
    entries = op.operator_bytes(hw.PREC_FP32) / 4
    fp32_nominal = 152 * 128 * 2 * 2.07e9
    ops_per_term = {"fp32": 2.0, "df64": 12.0, "fp64": 2.0}[top]
    achieved_ops = ops_per_term * entries * R / (tk["us"] / 1e6)
    plan = op.plan_stats()
    plan["padding_overhead"] = plan["multiplied"] / plan["entries"] - 1.0 if plan["entries"] else None
    roof = {"bound": "hbm", "achieved": tk["gbs"], "peak": peak, "unit": "GB/s", "frac": tk["gbs"] / peak,
            # the captured kernel's DRAM bytes, only when that kernel is the one reported here
            "traffic": ncu_traffic.get((kname, top)) if args.workload == "2d_ie_65536" and R == 64 else None,
            "compute": {"pipe": "fp64" if top == "fp64" else "fp32",
                        "ops_per_launch": ops_per_term * entries * R,
                        "achieved_tops": achieved_ops / 1e12,
                        "nominal_fp32_tops": fp32_nominal / 1e12,
                        "frac_of_nominal": achieved_ops / fp32_nominal if top != "fp64" else None,
                        "note": "each operator element feeds R FMAs: the pipe, not HBM, bounds this kernel",
                        # entries multiplied per column with the kernel's row and column padding
                        "plan": plan},
            "kernel": "%s<%s, %d> (one cooperative launch = one %d-vector matvec)" % (kname, ctype, rp, R),
            "bytes_per_launch": tk["bytes"], "launch_us": tk["us"], "launches": tk["launches"],
            "share_of_matvec_time": tk["ms"] / tot if tot else None,
            "peak_kind": (peak_kind + " (MEASURED_PEAKS.json hbm_gbs)") if peak_kind == "measured" else peak_kind,
            "per_precision": {k: {"launch_us": round(v["us"], 1), "GBs": round(v["gbs"], 1),
                                  "share": round(v["ms"] / tot, 3)} for k, v in kern.items()}}

    # ---- CPU baseline (one-GPU runs): the oracle on this host's cores, a bounded sample of the same workload
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        try:
            r = cpu_oracle_solves(wl, R, 1, 0, budget_s=20.0)
            cpu = {"value": 1.0 / r["t_solve"], "unit": "solves/s", "cores": r["cores"], "kind": "port",
                   "sample": "%d of the %d right-hand sides, each a full FP64 GMRES solve to 1e-%d (CPU oracle, "
                             "assembly %.2fs untimed, %d iterations, matvec %.1f ms)"
                             % (r["cols_per_step"], R, gtol, r["t_asm"], r["iters"], r["t_mv"] * 1e3)}
        except Exception as e:  # the GPU figures still print
            cpu = {"value": None, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": "CPU oracle failed: %s" % str(e)[:200]}

    # ---- assembly: plain NCA (timed again, warm) against learned proposals (the
    # shipped model; blocks the NCA stopping test rejects fall back to the plain
    # search), with each operator's error on the same exact dense rows
    def rows_err():
        y = op.matvec(xt)
        return float(np.linalg.norm(y[:nrow] - b_rows_xt) / np.linalg.norm(b_rows_xt))

    b_rows_xt = b_d[:nrow].cpu().numpy()
    asm = {}
    torch.cuda.synchronize()
    t0 = time.time()
    op.assemble(hw.ASSEMBLE_NCA)
    torch.cuda.synchronize()
    asm["plain"] = {"s": time.time() - t0, "storage_entries": op.storage_entries(), "dense_rows_rel_err": rows_err()}
    from h2weak_gb300 import learned
    params, calib, margin = learned.load()
    op.learn_set_model(params, calib, margin)
    op.learn_stats()
    torch.cuda.synchronize()
    t0 = time.time()
    op.assemble(hw.ASSEMBLE_LEARNED)
    torch.cuda.synchronize()
    t_l = time.time() - t0
    blocks, acc = op.learn_stats()
    asm["learned"] = {"s": t_l, "storage_entries": op.storage_entries(), "dense_rows_rel_err": rows_err(),
                      "blocks": blocks, "accepted": acc}
    asm["learned_speedup"] = asm["plain"]["s"] / t_l

    value = replica_throughput(K * R, world, ms_b)
    ms_solve_b = ms_b / K / R
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms_b / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": common_config(wl, N, nlev, R),
        "solver": "batched: FP32-operator inner GMRES (FP32 Krylov basis, FP64 Hessenberg and rotations, %d "
                  "columns in lockstep, one multi-vector matvec per step) + iterative refinement, residuals FP32 "
                  "at x0 then double-FP32 on the FP64 operator, later ones updated as r - A32 d under a "
                  "calibrated error bound; CUDA-graph Arnoldi loop" % R,
        "autotuned": {"multi_xw": tuned_xw, "multi_mix_ms": tuned_xw_ms,
                      "fp32_producer_warp": op.get_option(hw.OPT_PRODUCER_WARP),
                      "single_row_split": tuned_rs, "single_fp32_ms": tuned_rs_ms},
        "operator_mb": {"fp64": op.operator_bytes(hw.PREC_FP64) / 1e6, "fp32": op.operator_bytes(hw.PREC_FP32) / 1e6},
        "e2e": {"value": replica_throughput(K * R, world, ms_e2e), "unit": "solves/s", "h2d_bytes_per_step": 16 * N * R,
                "d2h_bytes_per_step": 8 * N * R},
        "gpu_launches": int(launches),
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(*win),
        "batched_mixed": {"ms_per_step": ms_b / K, "ms_per_solve": ms_solve_b, "outer": outer_b,
                          "inner_steps_total": inner_b, "max_resid": float(np.max(res_b)),
                          "max_fp64_resid": fp64_resid_b, "max_rel_err_vs_xtrue": err_b,
                          "dense_rows_rel_err_col0": dense_rows_err},
        "batched_fp64": {"ms_per_solve": ms_b64 / K / R, "iters": it_b64, "max_rel_err_vs_xtrue": err_b64},
        "single_mixed": {"ms_per_solve": ms_mixed / K, "outer": outer, "inner_total": inner, "resid": res_mixed,
                         "rel_err_vs_xtrue": err_mixed},
        "single_fp64": {"ms_per_solve": ms_fp64 / K, "iters": it64, "resid": res64, "rel_err_vs_xtrue": err_fp64},
        # same workload on both sides of each ratio: the R columns (batched), one column (single)
        "speedup_vs_plain_fp64": {"batched_mixed_over_batched_fp64": (ms_b64 / K / R) / ms_solve_b,
                                  "single_mixed_over_single_fp64": ms_fp64 / ms_mixed},
        "assembly_s": t_asm, "storage_entries": storage, "assembly": asm,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
