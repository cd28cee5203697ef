"""Command-line driver: build one operator and run products or solves on it,
printing one JSON line of timings (used for timing and ncu profiling outside
the benchmark).

    python -m h2weak_gb300.runner matvec [--rhs 64] [--precision fp32|fp64|df64] [--reps 3]
    python -m h2weak_gb300.runner solve  [--kind batched|batched_fp64|mixed|fp64] [--rhs 64] [--no-graph]

Problem options (defaults: 2D integral equation, 256^2 grid, nmax 64, NCA tol
1e-10): --dim --grid (points per axis) | --npts (uniform random) --leaf (points
per leaf axis, as the reference's drivers take it) --levels --form --choice
--tol --gtol --ir-residual fp64|df64.
"""
import argparse
import json
import time

import numpy as np

PREC = {"fp64": 0, "fp32": 1, "df64": 2}


def build_operator(a, hw, synth):
    if a.npts:
        N = a.npts
        op = hw.H2Operator(a.dim, a.form, a.choice, a.tol, a.levels, device=0)
        op.set_points(synth.uniform_points(synth.config_seed(5, 0), N, a.dim))
    else:
        N = a.grid ** a.dim
        levels = a.levels or hw.levels_for(a.dim, a.grid, a.leaf)
        op = hw.H2Operator(a.dim, a.form, a.choice, a.tol, levels, kernel_n=N, diag_n=2 * N if a.dim == 1 else N,
                           device=0)
        op.gen_grid(a.grid)
    op.build_tree()
    return op


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["matvec", "solve"])
    ap.add_argument("--dim", type=int, default=2)
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--npts", type=int, default=0)
    ap.add_argument("--leaf", type=int, default=8)
    ap.add_argument("--levels", type=int, default=0)
    ap.add_argument("--form", type=int, default=0)
    ap.add_argument("--choice", type=int, default=0)
    ap.add_argument("--tol", type=int, default=10)
    ap.add_argument("--gtol", type=int, default=10)
    ap.add_argument("--rhs", type=int, default=64)
    ap.add_argument("--precision", default="fp32", choices=sorted(PREC))
    ap.add_argument("--kind", default="batched", choices=["batched", "batched_fp64", "mixed", "fp64"])
    ap.add_argument("--ir-residual", default="df64", choices=["fp64", "df64"])
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--tensor", action="store_true", help="FP32 multi-vector products on the tensor cores")
    ap.add_argument("--no-dataflow", action="store_true", help="FP32 multi-vector products with grid barriers")
    a = ap.parse_args(argv)

    import torch
    import h2weak_gb300 as hw
    from h2weak_gb300 import synth
    op = build_operator(a, hw, synth)
    N = op.N
    torch.cuda.synchronize()
    t0 = time.time()
    op.assemble(hw.ASSEMBLE_NCA)
    torch.cuda.synchronize()
    out = {"what": a.what, "N": N, "assembly_s": time.time() - t0, "storage_entries": op.storage_entries()}
    if a.no_graph:
        op.set_option(hw.OPT_GRAPH, 0)
    if a.tensor:
        op.set_option(hw.OPT_TENSOR, 1)
    if a.no_dataflow:
        op.set_option(hw.OPT_DATAFLOW, 0)
    op.set_option(hw.OPT_IR_RESIDUAL, PREC[a.ir_residual])
    R = max(1, min(64, a.rhs))
    # column-major N x R blocks = rows of R x N tensors
    X = torch.from_numpy(np.stack([synth.normal(synth.config_seed(2, c), N) for c in range(R)], axis=0)).cuda()
    Y = torch.empty_like(X)
    B = torch.empty_like(X)
    torch.cuda.synchronize()
    if a.what == "solve":
        op.matvec_device(X.data_ptr(), B.data_ptr(), nrhs=R, precision=hw.PREC_FP64)
        torch.cuda.synchronize()

    def run():
        if a.what == "matvec":
            op.matvec_device(X.data_ptr(), Y.data_ptr(), nrhs=R, precision=PREC[a.precision])
            return None
        Y.fill_(1.0)
        torch.cuda.synchronize()  # the library runs on its own stream
        if a.kind == "batched":
            return op.gmres_ir_batch_device(B.data_ptr(), Y.data_ptr(), R, 20, 200, a.gtol)
        if a.kind == "batched_fp64":
            return op.gmres_batch_device(B.data_ptr(), Y.data_ptr(), R, 400, a.gtol)
        if a.kind == "mixed":
            return op.gmres_ir_device(B[0].data_ptr(), Y[0].data_ptr(), 20, 200, a.gtol)
        return op.gmres_device(B[0].data_ptr(), Y[0].data_ptr(), 500, a.gtol)

    run()
    torch.cuda.synchronize()
    t0 = time.time()
    res = None
    for _ in range(a.reps):
        res = run()
    torch.cuda.synchronize()
    out["ms_per_rep"] = (time.time() - t0) / max(a.reps, 1) * 1e3
    if res is not None:
        out["result"] = [float(np.max(r)) if hasattr(r, "tolist") else r for r in res]
    if R > 1:
        out["plan"] = op.plan_stats()
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
