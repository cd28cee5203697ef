"""Inner solves of the batched refinement on an FP32 Krylov basis (the
operator of those solves is FP32 already) against the FP64 basis: the same
tolerance on the true FP64 residual, outer steps within one, solution error
within 10x, with graphs and with the host-driven loop."""
import numpy as np
import pytest

from test_gpu_oracle import setup
from test_gpu_multi import CASES, rhs


def colerr(Y, R):
    return np.linalg.norm(Y - R, axis=0) / np.linalg.norm(R, axis=0)


@pytest.mark.gpu
@pytest.mark.parametrize("case,k,graph", [(CASES[1], 64, 1), (CASES[1], 7, 0), (CASES[4], 33, 1), (CASES[0], 16, 1)])
def test_f32_basis_inner_solves(gpu, case, k, graph):
    hw = gpu
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    op.set_option(hw.OPT_GRAPH, graph)
    assert op.get_option(hw.OPT_F32_BASIS) == 1
    XT = rhs(99, op.N, k)
    B = op.matvec(XT)
    tp = case[5]
    tol = 10.0 ** -tp
    X1, o1, i1, r1 = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=tp)
    op.set_option(hw.OPT_F32_BASIS, 0)
    X0, o0, i0, r0 = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=tp)
    op.set_option(hw.OPT_F32_BASIS, 1)
    assert np.all(r1 < tol) and np.all(r0 < tol)
    t1 = colerr(op.matvec(X1), B)
    assert np.all(t1 < tol), t1.max()
    assert abs(o1 - o0) <= 1, (o1, o0)
    e1, e0 = colerr(X1, XT), colerr(X0, XT)
    assert np.all(e1 <= 10 * e0 + 10 * tol), (e1.max(), e0.max())
