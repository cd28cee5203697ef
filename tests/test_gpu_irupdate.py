"""Refinement residual updating (r <- r - A32 d after an accurate residual):
the solvers reach the same tolerance on the TRUE FP64 residual, the reported
residual (||r|| plus the update's error bound) bounds the true one and stays
within the bound's budget (25 % of the tolerance) of it, and the update does
replace accurate products (taking r - A32 d from the inner solve's Arnoldi
relation, without a product)."""
import numpy as np
import pytest

from h2weak_gb300 import synth
from test_gpu_oracle import setup
from test_gpu_multi import CASES, rhs


def true_resid(op, B, X):
    R = B - op.matvec(X)
    if B.ndim == 1:
        return np.linalg.norm(R) / np.linalg.norm(B)
    return np.linalg.norm(R, axis=0) / np.linalg.norm(B, axis=0)


@pytest.mark.gpu
@pytest.mark.parametrize("tol_pow", [8, 10])
def test_ir_batch_residual_update(gpu, tol_pow):
    hw = gpu
    op, _ = setup(hw, CASES[1])
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    XT = rhs(81, N, 16)
    B = op.matvec(XT)
    tol = 10.0 ** -tol_pow
    op.set_option(hw.OPT_IR_UPDATE, 0)
    assert op.get_option(hw.OPT_IR_UPDATE) == 0
    op.profile(True)
    X0, o0, i0, r0 = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=tol_pow)
    acc_off = op.profile_multi(hw.PREC_FP64)[0]
    op.set_option(hw.OPT_IR_UPDATE, 1)
    op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=tol_pow)  # measures the FP32 error once
    op.profile(True)
    X1, o1, i1, r1 = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=tol_pow)
    acc_on = op.profile_multi(hw.PREC_FP64)[0]
    f32_on = op.profile_multi(hw.PREC_FP32)[0]
    op.profile(False)
    assert np.all(r0 < tol) and np.all(r1 < tol)
    t1 = true_resid(op, B, X1)
    assert np.all(t1 < tol), t1.max()
    assert np.all(t1 <= r1 * (1 + 1e-6)), (t1 - r1).max()
    assert np.all(r1 - t1 <= 0.3 * tol), (r1 - t1).max()
    assert abs(o1 - o0) <= 1 and abs(i1 - i0) <= 2, (o0, i0, o1, i1)
    for c in range(16):
        e0 = np.linalg.norm(X0[:, c] - XT[:, c]) / np.linalg.norm(XT[:, c])
        e1 = np.linalg.norm(X1[:, c] - XT[:, c]) / np.linalg.norm(XT[:, c])
        assert e1 <= 10 * e0 + 1e-12, (c, e1, e0)
    # one accurate residual per outer step without updating; with it only the
    # first tested residual needs the accurate product
    assert acc_off == o0
    if o0 >= 2 and tol_pow == 8:
        assert acc_on < acc_off, (acc_on, acc_off)
        # the updated residual came from the inner solve's Arnoldi relation: FP32
        # products = the residual at x0 + one per inner Arnoldi step, none for the update
        assert f32_on == 1 + i1, (f32_on, i1)
    print("accurate residual products: %d without updating, %d with" % (acc_off, acc_on))


@pytest.mark.gpu
def test_ir_batch_update_bounds_true_residual(gpu):
    """At tolerances near the FP64 floor the reported residual still bounds
    the true one (to the FP64 rounding of the check itself): updates stop
    where the accurate residual's own error approaches the tolerance."""
    hw = gpu
    op, _ = setup(hw, CASES[1])
    op.assemble(hw.ASSEMBLE_NCA)
    B = op.matvec(rhs(82, op.N, 4))
    for tp in (12, 13, 14):
        X, o, i, r = op.gmres_ir_batch(B, max_outer=6, inner_iter=100, tol_pow=tp)
        t = true_resid(op, B, X)
        assert np.all(t <= r * 1.5 + 1e-15), (tp, t, r)


@pytest.mark.gpu
def test_ir_single_residual_update(gpu):
    hw = gpu
    op, _ = setup(hw, CASES[2])
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    xt = synth.normal(synth.config_seed(83, 0), N)
    b = op.matvec(xt)
    op.set_option(hw.OPT_IR_UPDATE, 0)
    x0, o0, i0, r0 = op.gmres_ir(b, max_outer=20, inner_iter=100, tol_pow=10)
    op.set_option(hw.OPT_IR_UPDATE, 1)
    x1, o1, i1, r1 = op.gmres_ir(b, max_outer=20, inner_iter=100, tol_pow=10)
    assert r0 < 1e-10 and r1 < 1e-10
    t1 = true_resid(op, b, x1)
    assert t1 < 1e-10 and t1 <= r1 * (1 + 1e-6) and r1 - t1 <= 0.3e-10, (t1, r1)
    assert abs(o1 - o0) <= 1
    e0 = np.linalg.norm(x0 - xt) / np.linalg.norm(xt)
    e1 = np.linalg.norm(x1 - xt) / np.linalg.norm(xt)
    assert e1 <= 10 * e0 + 1e-12
