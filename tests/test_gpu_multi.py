"""Many right-hand sides: the multi-vector matvec against the oracle and the
single-vector path, and the batched (lockstep, per-column) GMRES and mixed
iterative refinement against the single-column solvers."""
import numpy as np
import pytest

from h2weak_gb300 import synth
from test_gpu_oracle import setup

CASES = [
    (1, 0, 8192, None, 7, 10, 1),
    (2, 0, 64, None, 4, 10, 1),
    (2, 1, 64, None, 4, 10, 0),
    (3, 0, 24, None, 3, 8, 0),
    (3, 1, 24, None, 3, 8, 1),
    (2, 1, None, 6000, 4, 8, 1),
]


def rhs(seed, N, k):
    return np.stack([synth.normal(synth.config_seed(seed, c), N) for c in range(k)], axis=1)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_multi_matvec_vs_oracle(gpu, case):
    """FP64 multi-vector product: every column within 1e-13 of the oracle's
    matvec on the same (imported) operator, for blocks of 16, 32, 64 and a
    ragged 64 + 6 split."""
    hw = gpu
    op, o = setup(hw, case)
    for nm in ["far_check", "far_charge", "ver_check", "ver_charge", "sn_row", "sn_col"]:
        p, v = o.csr(nm)
        op.import_list(nm, p, v)
    op.assemble(hw.ASSEMBLE_IMPORT)
    N = op.N
    X = rhs(70, N, 70)
    ref = {c: o.matvec(X[:, c]) for c in (0, 5, 17, 63, 69)}
    for k in (3, 20, 64, 70):
        Y = op.matvec(X[:, :k])
        assert Y.shape == (N, k)
        for c, yo in ref.items():
            if c < k:
                assert np.linalg.norm(Y[:, c] - yo) / np.linalg.norm(yo) <= 1e-13, (k, c)
    # every column against the single-vector GPU product
    Y = op.matvec(X[:, :40])
    for c in range(40):
        y1 = op.matvec(X[:, c])
        assert np.linalg.norm(Y[:, c] - y1) / np.linalg.norm(y1) <= 1e-14, c


@pytest.mark.gpu
@pytest.mark.parametrize("case", [CASES[1], CASES[4]])
def test_multi_matvec_fp32(gpu, case):
    """FP32 operator, FP32 accumulation: within 1e-5 of the FP64 product."""
    hw = gpu
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    X = rhs(71, op.N, 33)
    Y64 = op.matvec(X)
    Y32 = op.matvec(X, precision=hw.PREC_FP32)
    for c in range(33):
        assert np.linalg.norm(Y32[:, c] - Y64[:, c]) / np.linalg.norm(Y64[:, c]) < 1e-5, c


@pytest.mark.gpu
def test_multi_matvec_device_pointers(gpu):
    """Device-resident column-major blocks give the host path's result."""
    import torch
    hw = gpu
    op, _ = setup(hw, CASES[1])
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    X = rhs(72, N, 24)
    Yh = op.matvec(X)
    xd = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()  # row c = column c: column-major N x 24
    yd = torch.empty_like(xd)
    op.matvec_device(xd.data_ptr(), yd.data_ptr(), nrhs=24)
    torch.cuda.synchronize()
    Yd = yd.cpu().numpy().T
    # equal up to the order of atomically accumulated column splits
    for c in range(24):
        assert np.linalg.norm(Yd[:, c] - Yh[:, c]) / np.linalg.norm(Yh[:, c]) < 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("case", [CASES[0], CASES[1], CASES[4]])
def test_gmres_batch_matches_single(gpu, case):
    """Each column of the batched solve takes the single-column GMRES's
    iteration count (+-1) and reaches the same tolerance."""
    hw = gpu
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    XT = rhs(73, N, 5)
    B = op.matvec(XT)
    X, it, res = op.gmres_batch(B, max_iter=200, tol_pow=10)
    for c in range(5):
        x1, it1, res1 = op.gmres(B[:, c], max_iter=200, tol_pow=10)
        assert abs(int(it[c]) - it1) <= 1, (c, it[c], it1)
        assert res[c] < 1e-10
        e_b = np.linalg.norm(X[:, c] - XT[:, c]) / np.linalg.norm(XT[:, c])
        e_1 = np.linalg.norm(x1 - XT[:, c]) / np.linalg.norm(XT[:, c])
        assert e_b <= 10 * e_1 + 1e-12, (c, e_b, e_1)


@pytest.mark.gpu
def test_gmres_batch_mixed_convergence(gpu):
    """Columns converge at different steps (one is already solved by its
    initial guess, one is zero); the others keep iterating and stop on
    their own tolerance."""
    hw = gpu
    op, _ = setup(hw, CASES[1])
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    XT = rhs(74, N, 4)
    B = op.matvec(XT)
    B[:, 2] = 0.0
    X0 = np.ones((N, 4))
    X0[:, 1] = XT[:, 1]
    X0[:, 2] = 0.0
    X, it, res = op.gmres_batch(B, X0=X0, max_iter=200, tol_pow=10)
    assert it[1] <= 1 and it[2] == 0
    assert np.all(X[:, 2] == 0.0)
    for c in (0, 3):
        assert res[c] < 1e-10 and it[c] > 1
        assert np.linalg.norm(X[:, c] - XT[:, c]) / np.linalg.norm(XT[:, c]) < 1e-7


@pytest.mark.gpu
@pytest.mark.parametrize("k", [7, 64])
def test_gmres_ir_batch(gpu, k):
    """Mixed precision for k columns: every FP64 relative residual below
    1e-10, solution error within 10x of the FP64 single-column solve."""
    hw = gpu
    op, _ = setup(hw, CASES[1])
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    XT = rhs(75, N, k)
    B = op.matvec(XT)
    X, outer, inner, res = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=10)
    assert np.all(res < 1e-10), res.max()
    assert outer >= 1 and inner >= 1
    for c in (0, k - 1):
        x64, _, _ = op.gmres(B[:, c], max_iter=200, tol_pow=10)
        e_ir = np.linalg.norm(X[:, c] - XT[:, c]) / np.linalg.norm(XT[:, c])
        e_64 = np.linalg.norm(x64 - XT[:, c]) / np.linalg.norm(XT[:, c])
        assert e_ir <= 10 * e_64 + 1e-12, (c, e_ir, e_64)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [CASES[0], CASES[2], CASES[4]])
def test_multi_matvec_df64(gpu, case):
    """Double-FP32 products on the FP64 operator: within 1e-12 of the FP64
    product per column (FP32 alone is ~1e-7), including one right-hand side."""
    hw = gpu
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    X = rhs(76, op.N, 40)
    Y64 = op.matvec(X)
    Ydf = op.matvec(X, precision=hw.PREC_DF64)
    for c in range(40):
        assert np.linalg.norm(Ydf[:, c] - Y64[:, c]) / np.linalg.norm(Y64[:, c]) < 1e-12, c
    y1 = op.matvec(X[:, 3], precision=hw.PREC_DF64)
    assert np.linalg.norm(y1 - Y64[:, 3]) / np.linalg.norm(Y64[:, 3]) < 1e-12


@pytest.mark.gpu
def test_gmres_ir_batch_df64_residuals(gpu):
    """Refinement residuals in double-FP32: same tolerance reached, solution
    error within 10x of the FP64-residual refinement."""
    hw = gpu
    op, _ = setup(hw, CASES[1])
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    XT = rhs(77, N, 16)
    B = op.matvec(XT)
    X64, o64, i64, r64 = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=10)
    op.set_option(hw.OPT_IR_RESIDUAL, hw.PREC_DF64)
    assert op.get_option(hw.OPT_IR_RESIDUAL) == hw.PREC_DF64
    Xdf, odf, idf, rdf = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=10)
    assert np.all(rdf < 1e-10)
    # the FP64 residual of the DF64-refined solution
    R = B - op.matvec(Xdf)
    for c in range(16):
        assert np.linalg.norm(R[:, c]) / np.linalg.norm(B[:, c]) < 1e-10
        e_df = np.linalg.norm(Xdf[:, c] - XT[:, c]) / np.linalg.norm(XT[:, c])
        e_64 = np.linalg.norm(X64[:, c] - XT[:, c]) / np.linalg.norm(XT[:, c])
        assert e_df <= 10 * e_64 + 1e-12, (c, e_df, e_64)
