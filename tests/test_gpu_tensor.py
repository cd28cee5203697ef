"""FP32 multi-vector product on the tensor cores (tcgen05 TF32 MMAs on
hi/lo-split operands) against the FP64 product and the FP32 FMA kernel, on
1D/2D/3D operators of both forms, blocks of 16/32/64 columns and a ragged
split, cooperative and per-phase launches, and inside the batched mixed
solver (graph and host loop)."""
import numpy as np
import pytest

from test_gpu_oracle import setup
from test_gpu_multi import CASES, rhs


def colerr(Y, R):
    return np.linalg.norm(Y - R, axis=0) / np.linalg.norm(R, axis=0)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_tensor_product_fp32_accuracy(gpu, case):
    hw = gpu
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    assert op.get_option(hw.OPT_TENSOR) == 0
    op.set_option(hw.OPT_TENSOR, 1)
    for k in (7, 16, 32, 64, 70):
        X = rhs(90 + k, op.N, k)
        Y64 = op.matvec(X)
        Ytc = op.matvec(X, precision=hw.PREC_FP32)
        op.set_option(hw.OPT_TENSOR, 0)
        Yfma = op.matvec(X, precision=hw.PREC_FP32)
        op.set_option(hw.OPT_TENSOR, 1)
        e_tc, e_fma = colerr(Ytc, Y64), colerr(Yfma, Y64)
        # FP32-level accuracy: within 1e-5 and within a few times the FMA kernel's error
        assert np.all(e_tc < 1e-5), (k, e_tc.max())
        assert e_tc.max() <= 8 * e_fma.max() + 1e-7, (k, e_tc.max(), e_fma.max())
        assert not np.array_equal(Ytc, Yfma)  # a different kernel ran


@pytest.mark.gpu
def test_tensor_product_phased_launch(gpu):
    hw = gpu
    op, _ = setup(hw, CASES[4])
    op.assemble(hw.ASSEMBLE_NCA)
    op.set_option(hw.OPT_TENSOR, 1)
    X = rhs(97, op.N, 64)
    Y64 = op.matvec(X)
    Yc = op.matvec(X, precision=hw.PREC_FP32)
    op.set_option(hw.OPT_COOP, 0)
    Yp = op.matvec(X, precision=hw.PREC_FP32)
    op.set_option(hw.OPT_COOP, 1)
    assert np.all(colerr(Yp, Y64) < 1e-5)
    # same kernel body, different target-to-CTA assignment: equal up to atomics order
    assert np.all(colerr(Yp, Yc) < 1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [1, 0])
def test_tensor_in_batched_mixed_solve(gpu, graph):
    hw = gpu
    op, _ = setup(hw, CASES[1])
    op.assemble(hw.ASSEMBLE_NCA)
    op.set_option(hw.OPT_GRAPH, graph)
    op.set_option(hw.OPT_IR_RESIDUAL, hw.PREC_DF64)
    op.set_option(hw.OPT_TENSOR, 1)
    N = op.N
    XT = rhs(98, N, 64)
    B = op.matvec(XT)
    X, outer, inner, res = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=10)
    assert np.all(res < 1e-10)
    t = colerr(op.matvec(X), B)
    assert np.all(t < 1e-10), t.max()
    op.set_option(hw.OPT_TENSOR, 0)
    Xf, of, i_f, rf = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=10)
    assert abs(outer - of) <= 1 and abs(inner - i_f) <= 3, (outer, inner, of, i_f)
    e_tc, e_f = colerr(X, XT), colerr(Xf, XT)
    assert e_tc.max() <= 10 * e_f.max() + 1e-12
