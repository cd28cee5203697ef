"""GPU against the CPU oracle on seeded cases in all dimensions and both
forms (sizes the oracle assembles in seconds), including the 1D
semi-nested form whose UV pivots only the oracle exports."""
import numpy as np
import pytest

from h2weak_gb300 import synth

CASES = [
    # dim, form, grid n (or None), npts, nlevels, tol, choice
    (1, 0, 8192, None, 7, 10, 1),
    (1, 1, 8192, None, 7, 10, 1),
    (1, 1, 4096, None, 6, 10, 0),
    (2, 0, 64, None, 4, 10, 1),
    (2, 1, 64, None, 4, 10, 0),
    (3, 0, 24, None, 3, 8, 0),
    (3, 1, 24, None, 3, 8, 1),
    (2, 1, None, 6000, 4, 8, 1),
    (3, 1, None, 6000, 2, 8, 0),
]


def setup(hw, case):
    from oracle import Oracle
    dim, form, n, npts, nlev, tol, ch = case
    op = hw.H2Operator(dim, form, ch, tol, nlev, device=0)
    if n is None:
        op.set_points(synth.uniform_points(synth.config_seed(50 + dim, form), npts, dim))
    else:
        op.gen_grid(n)
    N = op.N
    op2 = hw.H2Operator(dim, form, ch, tol, nlev, kernel_n=N, diag_n=2 * N if dim == 1 else N, device=0)
    op2.set_points(op.points())
    op2.build_tree()
    o = Oracle(dim, form, op.points(), nlev, tol, ch, N, 2 * N if dim == 1 else N)
    return op2, o


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_vs_oracle(gpu, case):
    hw = gpu
    op, o = setup(hw, case)
    N, dim, form = op.N, case[0], case[1]
    names = ["far_check", "far_charge", "ver_check", "ver_charge", "sn_row", "sn_col"]
    for nm in names:
        p, v = o.csr(nm)
        op.import_list(nm, p, v)
    op.assemble(hw.ASSEMBLE_IMPORT)
    assert op.storage_entries() == o.memory()
    x = synth.normal(synth.config_seed(60, 0), N)
    y, yo = op.matvec(x), o.matvec(x)
    assert np.linalg.norm(y - yo) / np.linalg.norm(yo) <= 1e-13
    # own NCA: same storage when every entry is IEEE-exact
    op.assemble(hw.ASSEMBLE_NCA)
    if (dim, case[6]) in {(1, 1), (2, 1), (3, 0)}:
        assert op.storage_entries() == o.memory()
    y2 = op.matvec(x)
    yd = o.dense_matvec(x) if N <= 16384 else None
    if yd is not None:
        e_o = np.linalg.norm(yo - yd) / np.linalg.norm(yd)
        e_g = np.linalg.norm(y2 - yd) / np.linalg.norm(yd)
        assert e_g <= 10 * e_o + 1e-14, (e_g, e_o)


@pytest.mark.gpu
def test_gpu_fp32_matvec_close_to_fp64(gpu):
    hw = gpu
    op, o = setup(hw, (2, 0, 64, None, 4, 10, 1))
    op.assemble(hw.ASSEMBLE_NCA)
    x = synth.normal(synth.config_seed(61, 0), op.N)
    y64 = op.matvec(x)
    y32 = op.matvec(x, precision=hw.PREC_FP32)
    assert np.linalg.norm(y32 - y64) / np.linalg.norm(y64) < 1e-5


@pytest.mark.gpu
def test_gpu_linearity_and_multi_rhs(gpu):
    hw = gpu
    op, o = setup(hw, (3, 0, 24, None, 3, 8, 1))
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    x1 = synth.normal(synth.config_seed(62, 0), N)
    x2 = synth.normal(synth.config_seed(62, 1), N)
    y1, y2 = op.matvec(x1), op.matvec(x2)
    y12 = op.matvec(2.0 * x1 - 3.0 * x2)
    assert np.linalg.norm(y12 - (2.0 * y1 - 3.0 * y2)) / np.linalg.norm(y12) < 1e-13
    Y = op.matvec(np.stack([x1, x2], axis=1))
    assert np.allclose(Y[:, 0], y1, rtol=0, atol=1e-14 * np.abs(y1).max())
    assert np.allclose(Y[:, 1], y2, rtol=0, atol=1e-14 * np.abs(y2).max())


@pytest.mark.gpu
def test_gpu_gmres_ir_reaches_tolerance(gpu):
    hw = gpu
    op, o = setup(hw, (2, 0, 64, None, 4, 10, 0))
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    xt = synth.normal(synth.config_seed(63, 0), N)
    b = op.dense_matvec(xt)
    x, outer, inner, res = op.gmres_ir(b, max_outer=20, inner_iter=100, tol_pow=10)
    assert res < 1e-10
    x64, it, res64 = op.gmres(b, max_iter=200, tol_pow=10)
    e_ir = np.linalg.norm(x - xt) / np.linalg.norm(xt)
    e_64 = np.linalg.norm(x64 - xt) / np.linalg.norm(xt)
    assert e_ir <= 10 * e_64 + 1e-12, (e_ir, e_64)
