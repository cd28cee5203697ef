"""Dataflow launch of the multi-vector products (targets wait for the
targets producing their workspace rows, no grid barriers) against the
barrier-phased launch and the FP64 product, for FP32, FP64 and double-FP32, on 1D/2D/3D operators of both
forms and blocks of 7/16/32/64 columns, and inside the batched mixed solve."""
import numpy as np
import pytest

from test_gpu_oracle import setup
from test_gpu_multi import CASES, rhs


def colerr(Y, R):
    return np.linalg.norm(Y - R, axis=0) / np.linalg.norm(R, axis=0)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_dataflow_product(gpu, case):
    hw = gpu
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    assert op.get_option(hw.OPT_DATAFLOW) == 1
    for k in (7, 16, 32, 64):
        X = rhs(110 + k, op.N, k)
        Y64 = op.matvec(X)
        Yf = op.matvec(X, precision=hw.PREC_FP32)
        op.set_option(hw.OPT_DATAFLOW, 0)
        Yb = op.matvec(X, precision=hw.PREC_FP32)
        op.set_option(hw.OPT_DATAFLOW, 1)
        # same per-target arithmetic; only the order of atomically accumulated column splits differs
        assert np.all(colerr(Yf, Yb) < 1e-6), (k, colerr(Yf, Yb).max())
        assert np.all(colerr(Yf, Y64) < 1e-5), (k, colerr(Yf, Y64).max())
        # FP64 and double-FP32 products on the dataflow launch against the barrier launch
        Ydf = op.matvec(X, precision=hw.PREC_DF64)
        op.set_option(hw.OPT_DATAFLOW, 0)
        Y64b = op.matvec(X)
        Ydfb = op.matvec(X, precision=hw.PREC_DF64)
        op.set_option(hw.OPT_DATAFLOW, 1)
        assert np.all(colerr(Y64, Y64b) < 1e-14), (k, colerr(Y64, Y64b).max())
        assert np.all(colerr(Ydf, Ydfb) < 1e-13), (k, colerr(Ydf, Ydfb).max())
        assert np.all(colerr(Ydf, Y64) < 1e-12), (k, colerr(Ydf, Y64).max())
    # repeated launches give the same result (counters reset per launch)
    X = rhs(120, op.N, 64)
    Y1 = op.matvec(X, precision=hw.PREC_FP32)
    Y2 = op.matvec(X, precision=hw.PREC_FP32)
    assert np.all(colerr(Y1, Y2) < 1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_producer_warp_product(gpu, case):
    """FP32 multi-vector product of the warp-specialised dataflow kernel
    (producer warp + bulk copies) against the kernel whose warps all stage
    and multiply, for blocks of 7/16/32/64 columns (RP 16, 32 and 64), FP32
    and FP64 outputs, and repeated launches."""
    hw = gpu
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    assert op.get_option(hw.OPT_PRODUCER_WARP) == 1
    for k in (7, 16, 32, 64):
        X = rhs(140 + k, op.N, k)
        Y64 = op.matvec(X)
        Yw = op.matvec(X, precision=hw.PREC_FP32)
        op.set_option(hw.OPT_PRODUCER_WARP, 0)
        Yo = op.matvec(X, precision=hw.PREC_FP32)
        op.set_option(hw.OPT_PRODUCER_WARP, 1)
        # the same per-target sums; split-K parts and atomics may add in another order
        assert np.all(colerr(Yw, Yo) < 1e-6), (k, colerr(Yw, Yo).max())
        assert np.all(colerr(Yw, Y64) < 1e-5), (k, colerr(Yw, Y64).max())
    X = rhs(150, op.N, 64)
    Y1 = op.matvec(X, precision=hw.PREC_FP32)
    Y2 = op.matvec(X, precision=hw.PREC_FP32)
    assert np.all(colerr(Y1, Y2) < 1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [1, 0])
def test_dataflow_in_batched_mixed_solve(gpu, graph):
    hw = gpu
    op, _ = setup(hw, CASES[1])
    op.assemble(hw.ASSEMBLE_NCA)
    op.set_option(hw.OPT_GRAPH, graph)
    op.set_option(hw.OPT_IR_RESIDUAL, hw.PREC_DF64)
    op.set_option(hw.OPT_DATAFLOW, 1)
    XT = rhs(121, op.N, 64)
    B = op.matvec(XT)
    X, outer, inner, res = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=10)
    assert np.all(res < 1e-10)
    t = colerr(op.matvec(X), B)
    assert np.all(t < 1e-10), t.max()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_dataflow_single_vector_product(gpu, case):
    """One right-hand side (the single-vector stream) on the dataflow launch
    against the barrier launch, FP64 and FP32."""
    hw = gpu
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    x = rhs(130, op.N, 1)[:, 0]
    y64 = op.matvec(x)
    y32 = op.matvec(x, precision=hw.PREC_FP32)
    op.set_option(hw.OPT_DATAFLOW, 0)
    b64 = op.matvec(x)
    b32 = op.matvec(x, precision=hw.PREC_FP32)
    op.set_option(hw.OPT_DATAFLOW, 1)
    assert np.linalg.norm(y64 - b64) / np.linalg.norm(b64) < 1e-14
    assert np.linalg.norm(y32 - b32) / np.linalg.norm(b32) < 1e-6
