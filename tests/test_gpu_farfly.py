"""The far-field M2L evaluated during the product (H2W_OPT_FAR_ON_THE_FLY)
against the stored operator on the same pivots: FP64 products equal to
1e-13 (the same entries, summed in another order), FP32 products within FP32
accuracy, the double-FP32 form within 1e-12, GMRES and the mixed-precision
solve (FP64 or double-FP32 residuals) reaching the same tolerance;
the storage count stays the reference's; multi-vector products refuse."""
import numpy as np
import pytest

from h2weak_gb300 import synth

CASES = [
    # dim, choice, grid n (or None), npts, nlevels, tol
    (3, 1, None, 20000, 3, 10),
    (3, 0, 20, None, 3, 8),
    (2, 0, 64, None, 4, 10),
    (2, 1, None, 12000, 4, 8),
]


def relerr(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def pair(hw, case):
    dim, ch, n, npts, nl, tol = case
    ops = []
    for fly in (0, 1):
        op = hw.H2Operator(dim, hw.FORM_NESTED, ch, tol, nl, device=0)
        if n is None:
            op.set_points(synth.uniform_points(synth.config_seed(5, npts), npts, dim))
        else:
            op.gen_grid(n)
        op.build_tree()
        op.set_option(hw.OPT_FAR_ON_THE_FLY, fly)
        ops.append(op)
    ops[0].assemble(hw.ASSEMBLE_NCA)
    for nm in ("far_check", "far_charge", "ver_check", "ver_charge"):
        p, v = ops[0].get_list(nm)
        ops[1].import_list(nm, p, v)
    ops[1].assemble(hw.ASSEMBLE_IMPORT)
    return ops


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_far_on_the_fly_matches_stored(gpu, case):
    hw = gpu
    st, fl = pair(hw, case)
    assert fl.get_option(hw.OPT_FAR_ON_THE_FLY) == 1
    assert fl.storage_entries() == st.storage_entries()
    assert fl.operator_bytes() < st.operator_bytes()
    for k in range(2):
        x = synth.normal(synth.config_seed(74, k), st.N)
        y = st.matvec(x)
        assert relerr(fl.matvec(x), y) <= 1e-13, k
        assert relerr(fl.matvec(x, precision=hw.PREC_FP32), y) <= 2e-5, k
    xt = synth.normal(synth.config_seed(75, 0), st.N)
    b = st.dense_matvec(xt)
    x1, it1, r1 = st.gmres(b, tol_pow=10)
    x2, it2, r2 = fl.gmres(b, tol_pow=10)
    assert abs(it1 - it2) <= 1 and r2 < 1e-10
    assert relerr(x2, xt) <= 10 * relerr(x1, xt) + 1e-13
    xm, outer, inner, rm = fl.gmres_ir(b, max_outer=20, inner_iter=200, tol_pow=10)
    assert rm < 1e-10
    assert relerr(st.matvec(xm), b) < 1e-10
    # the FP64-accurate double-FP32 form of the far field (FP64 where it has none)
    x = synth.normal(synth.config_seed(74, 2), st.N)
    assert relerr(fl.matvec(x, precision=hw.PREC_DF64), st.matvec(x)) <= 1e-12
    fl.set_option(hw.OPT_IR_RESIDUAL, hw.PREC_DF64)
    xd, outer, inner, rd = fl.gmres_ir(b, max_outer=20, inner_iter=200, tol_pow=10)
    assert rd < 1e-10
    assert relerr(st.matvec(xd), b) < 1e-10
    with pytest.raises(hw.H2WError):
        fl.matvec(np.stack([x1, x2], axis=1))
