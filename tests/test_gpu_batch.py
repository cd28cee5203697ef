"""Many independent problems of uneven size (2D, uniform random points per
seed, both kernel choices, different tree depths) run together: one
cooperative launch per product over all problems against each problem's own
product, and the lockstep solvers against each problem's own GMRES."""
import numpy as np
import pytest

from h2weak_gb300 import synth


def problems(hw, sizes, tol=8):
    ops = []
    for i, n in enumerate(sizes):
        nl = max(1, int(np.ceil(np.log(n / 64.0) / np.log(4.0))))
        op = hw.H2Operator(2, hw.FORM_NESTED, i % 2, tol, nl, device=0)
        op.set_points(synth.uniform_points(synth.config_seed(4, i), n, 2))
        op.build_tree()
        op.assemble(hw.ASSEMBLE_NCA)
        ops.append(op)
    return ops


SIZES = [1024, 3000, 1500, 8192, 2048, 5000, 1100, 4096]


@pytest.mark.gpu
def test_batch_matvec_matches_each_problem(gpu):
    hw = gpu
    ops = problems(hw, SIZES)
    B = hw.Batch(ops)
    assert B.N == sum(SIZES)
    x = synth.normal(synth.config_seed(87, 0), B.N)
    for prec, tol in ((hw.PREC_FP64, 1e-14), (hw.PREC_FP32, 1e-6)):
        y = B.matvec(x, precision=prec)
        for op, xs, ys in zip(ops, B.split(x), B.split(y)):
            ye = op.matvec(xs, precision=prec)
            assert np.linalg.norm(ys - ye) / np.linalg.norm(ye) < tol
    y2 = B.matvec(x)  # a second call on the same state
    assert np.allclose(y2, B.matvec(x), rtol=0, atol=1e-13 * np.abs(y2).max())


@pytest.mark.gpu
def test_batch_gmres_matches_each_problem(gpu):
    hw = gpu
    ops = problems(hw, SIZES)
    B = hw.Batch(ops)
    xt = synth.normal(synth.config_seed(88, 0), B.N)
    b = B.matvec(xt)
    x, it, res = B.gmres(b, max_iter=200, tol_pow=10)
    assert np.all(res < 1e-10)
    for p, (op, bs, xs, xts) in enumerate(zip(ops, B.split(b), B.split(x), B.split(xt))):
        x1, it1, _ = op.gmres(bs, max_iter=200, tol_pow=10)
        assert abs(int(it[p]) - it1) <= 1, (p, it[p], it1)
        e_b = np.linalg.norm(xs - xts) / np.linalg.norm(xts)
        e_1 = np.linalg.norm(x1 - xts) / np.linalg.norm(xts)
        assert e_b <= 10 * e_1 + 1e-12, (p, e_b, e_1)
    # mixed precision for every problem
    x, outer, inner, res = B.gmres_ir(b, max_outer=20, inner_iter=100, tol_pow=10)
    assert np.all(res < 1e-10) and outer >= 1
    for op, bs, xs in zip(ops, B.split(b), B.split(x)):
        r = bs - op.matvec(xs)
        assert np.linalg.norm(r) / np.linalg.norm(bs) < 1e-10
