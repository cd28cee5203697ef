"""GPU parity against the golden fixtures produced by the reference's own
code: tree lists bit-exact, NCA pivots (bit-exact for kernels built from
IEEE-exact operations; agreement rate reported for log kernels, whose CUDA
and glibc log may differ in the last bit), storage counts, matvec on the
reference's own compressed operator (imported pivots) to <= 1e-13 relative,
and GMRES iterations within +-1."""
import numpy as np
import pytest

from conftest import golden_names, load_golden

IEEE = {(1, 1), (2, 1), (3, 0)}  # (dim, choice) whose entries use only + - * / sqrt
LIST_NAMES = ["far_check", "far_charge", "ver_check", "ver_charge", "sn_row", "sn_col"]
MATVEC_RTOL = 1e-13
# g2d_n_snap (2D RBF, random points with about a third of their coordinates on
# the split planes): the product on this operator cancels strongly, so its
# rounding depends on the summation order. Summing every block product of the
# CPU oracle in reverse order (the same operator, bit for bit) moves its result
# 1.24e-13 from the reference's, against 3e-16 on every other fixture
# (test_oracle_golden.py::test_product_dependence_on_summation_order); the GPU
# sums in its own order and measured 1.66e-13 on a GB300, with pivots and
# storage bit-exact.
MATVEC_RTOL_CASE = {"g2d_n_snap": 2.5e-13}


def make_op(hw, g):
    N, dim = g["N"], g["dim"]
    op = hw.H2Operator(dim, g["form"], g["choice"], g["tol_pow"], g["nlevels"], kernel_n=N,
                       diag_n=2 * N if dim == 1 else N, device=0)
    op.set_points(g["points"])
    op.build_tree()
    return op


def relerr(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_gpu_nca_assembly_vs_reference(gpu, name):
    hw = gpu
    g = load_golden(name)
    op = make_op(hw, g)
    for nm in ["charge", "nbr", "il"] + (["isvertex"] if g["form"] != 2 else []):
        p, v = op.get_list(nm)
        assert np.array_equal(p, g[nm + "_ptr"]) and np.array_equal(v, g[nm + "_val"]), nm
    op.assemble(hw.ASSEMBLE_NCA)
    exact = (g["dim"], g["choice"]) in IEEE
    names = LIST_NAMES if g["dim"] > 1 else ["far_check", "far_charge"]
    agree, total = 0, 0
    for nm in names:
        p, v = op.get_list(nm)
        gp, gv = g[nm + "_ptr"], g[nm + "_val"]
        if exact:
            assert np.array_equal(p, gp) and np.array_equal(v, gv), nm
        for i in range(len(gp) - 1):
            a, b = v[p[i]:p[i + 1]], gv[gp[i]:gp[i + 1]]
            total += 1
            agree += int(np.array_equal(a, b))
    if exact:
        assert op.storage_entries() == g["memory"][0]
    else:
        assert agree >= 0.9 * total, (agree, total)
        assert abs(op.storage_entries() - g["memory"][0]) <= 0.01 * g["memory"][0]
    y = op.matvec(g["vecs"][0])
    if exact:
        assert relerr(y, g["matvec"][0]) <= MATVEC_RTOL_CASE.get(name, MATVEC_RTOL)
    # against the exact dense product: the compression error of the reference
    ref_err = relerr(g["matvec"][0], g["dense_matvec"])
    assert relerr(y, g["dense_matvec"]) <= max(10 * ref_err, 1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in golden_names() if not n.startswith("g1d_sn")])
def test_gpu_matvec_on_reference_operator(gpu, name):
    """Import the reference's pivots: the GPU matvec then applies the same
    compressed operator, to <= 1e-13 relative."""
    hw = gpu
    g = load_golden(name)
    op = make_op(hw, g)
    names = LIST_NAMES if g["dim"] > 1 else ["far_check", "far_charge"]
    for nm in names:
        op.import_list(nm, g[nm + "_ptr"], g[nm + "_val"])
    op.assemble(hw.ASSEMBLE_IMPORT)
    assert op.storage_entries() == g["memory"][0]
    for k in range(2):
        assert relerr(op.matvec(g["vecs"][k]), g["matvec"][k]) <= MATVEC_RTOL_CASE.get(name, MATVEC_RTOL)


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_gpu_gmres_vs_reference(gpu, name):
    hw = gpu
    g = load_golden(name)
    op = make_op(hw, g)
    op.assemble(hw.ASSEMBLE_NCA)
    x, it, res = op.gmres(g["gmres_rhs"], max_iter=500, tol_pow=g["gtol"])
    it_ref, res_ref, err_ref = g["gmres_stats"]
    assert abs(it - int(it_ref)) <= 1, (it, it_ref)
    assert res < 10.0 ** (-g["gtol"])
    err = np.linalg.norm(x - g["xtrue"]) / np.linalg.norm(g["xtrue"])
    assert err <= 10 * err_ref + 1e-13, (err, err_ref)
