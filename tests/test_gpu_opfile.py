"""Operator files (h2w_save_operator / h2w_open_operator): an assembled
operator written to disk and opened in a new handle gives bitwise the same
products and solver results, in every form; a damaged file is refused.
And the GPU error tooling: h2w_total_error against the reference's own
compressed and dense products (compute_total_error,
3D/codes/HODLR3Dtree.hpp:2645-2662)."""
import numpy as np
import pytest

from conftest import load_golden
from h2weak_gb300 import synth


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1, 2])
def test_operator_file_round_trip(gpu, tmp_path, form):
    hw = gpu
    op = hw.H2Operator(2, form, 1, 10, 4, device=0)
    op.gen_grid(64)
    op.build_tree()
    op.assemble(hw.ASSEMBLE_NCA)
    path = str(tmp_path / "op.h2w")
    op.save(path)
    op2 = hw.H2Operator.open(path, device=0)
    assert op2.N == op.N and op2.form == form
    assert op2.storage_entries() == op.storage_entries()
    x = synth.normal(synth.config_seed(80, form), op.N)
    assert np.array_equal(op2.matvec(x), op.matvec(x))
    assert np.array_equal(op2.matvec(x, precision=hw.PREC_FP32), op.matvec(x, precision=hw.PREC_FP32))
    b = op.dense_matvec(x)
    x1, it1, r1 = op.gmres(b, tol_pow=10)
    x2, it2, r2 = op2.gmres(b, tol_pow=10)
    assert it1 == it2 and np.array_equal(x1, x2)
    # one flipped byte: refused
    raw = bytearray(open(path, "rb").read())
    raw[len(raw) // 2] ^= 0x40
    bad = str(tmp_path / "bad.h2w")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(hw.H2WError):
        hw.H2Operator.open(bad, device=0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["g2d_n_rand", "g3d_sn_ie", "g1d_n_rbf", "g2d_nn_rbf"])
def test_total_error_vs_reference(gpu, name):
    """On the reference's own pivots the compressed operator is the
    reference's: the error against the dense product equals the one of the
    reference's products, every row and sampled rows."""
    hw = gpu
    g = load_golden(name)
    N, dim = g["N"], g["dim"]
    op = hw.H2Operator(dim, g["form"], g["choice"], g["tol_pow"], g["nlevels"], kernel_n=N,
                       diag_n=2 * N if dim == 1 else N, device=0)
    op.set_points(g["points"])
    op.build_tree()
    names = ["far_check", "far_charge", "ver_check", "ver_charge", "sn_row", "sn_col"] if dim > 1 else \
        ["far_check", "far_charge"]
    for nm in names:
        op.import_list(nm, g[nm + "_ptr"], g[nm + "_val"])
    op.assemble(hw.ASSEMBLE_IMPORT)
    x = g["vecs"][0]
    ref = np.linalg.norm(g["dense_matvec"] - g["matvec"][0]) / np.linalg.norm(g["dense_matvec"])
    e = op.total_error(x)
    assert abs(e - ref) <= 1e-3 * ref + 1e-15, (e, ref)
    rows = np.array([(i * N) // 256 for i in range(256)])
    ref_s = np.linalg.norm(g["dense_matvec"][rows] - g["matvec"][0][rows]) / np.linalg.norm(g["dense_matvec"][rows])
    es = op.total_error(x, nrows=256)
    assert abs(es - ref_s) <= 1e-3 * ref_s + 1e-15, (es, ref_s)
    # the mirror of the reference's tree object: the error of the last mat_vec_prod
    init = hw.initialisation(g["n_param"], g["nlevels"], g["leaf"], 1, g["tol_pow"], g["choice"], dim=dim,
                             form=g["form"], points=g["points"])
    init.tree_initialisation(skeleton={nm: (g[nm + "_ptr"], g[nm + "_val"]) for nm in names})
    init.mat_vec_prod(x)
    assert abs(init.K.compute_total_error() - ref) <= 1e-3 * ref + 1e-15
