"""The complex Helmholtz kernel (the reference's USE_Helm build, choice 2:
exp(iR)/(4 pi) off the diagonal, 500 sqrt(N) on it, 3D/codes/kernel.hpp:132-144).

Parity against the reference's own outputs runs through the golden fixtures
g3d_*_helm* (tests/test_gpu_golden.py: pivots, storage, the product on the
reference's pivots to <= 1e-13, GMRES iterations +-1; tests/test_gpu_configs.py:
the dense product). This file adds what the fixtures do not cover: a larger
problem against the exact dense product, complex linearity of the product,
and the refusal of the entry points that are real-only."""
import numpy as np
import pytest

from h2weak_gb300 import synth


def relerr(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def cvec(seed, n):
    return synth.normal(synth.config_seed(95, seed), n) + 1j * synth.normal(synth.config_seed(96, seed), n)


def helm_op(hw, n, nlev, tol, form=0, seed=7):
    op = hw.H2Operator(3, form, hw.KERNEL_HELMHOLTZ, tol, nlev, device=0)
    op.set_points(synth.uniform_points(synth.config_seed(97, seed), n, 3))
    op.build_tree()
    op.assemble(hw.ASSEMBLE_NCA)
    return op


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_helmholtz_product_against_dense_rows(gpu, form):
    """3D Helmholtz on 20 000 random points, 3 levels, tol 1e-8: the compressed
    product agrees with the exact dense product (sampled rows) to the NCA
    tolerance, and is linear over the complex numbers."""
    hw = gpu
    n = 20000
    op = helm_op(hw, n, 3, 8, form)
    x = cvec(0, n)
    y = op.matvec(x)
    rows = np.arange(0, n, 37)
    yd = np.concatenate([op.dense_matvec(x, row0=int(r), nrows=1) for r in rows[:64]])
    err = relerr(y[rows[:64]], yd)
    assert err < 1e-7, err
    a = 0.3 - 1.7j
    x2 = cvec(1, n)
    y2 = op.matvec(x2)
    assert relerr(op.matvec(a * x + x2), a * y + y2) < 1e-13
    # the entries are symmetric (K(i,j) = K(j,i), not Hermitian): x^T A z = z^T A x
    assert abs(x2 @ y - x @ y2) <= 1e-9 * abs(x @ y2)


@pytest.mark.gpu
def test_helmholtz_gmres_solves(gpu):
    """GMRES on the complex operator reaches its stopping test (the reference's
    |s(i+1)| / ||b||); with H2W_OPT_COMPLEX_ARNOLDI the solution is accurate."""
    hw = gpu
    n = 8000
    op = helm_op(hw, n, 2, 10)
    xt = cvec(2, n)
    b = op.matvec(xt)
    x, it, res = op.gmres(b, max_iter=200, tol_pow=10)
    assert res < 1e-10 and 1 <= it <= 200
    assert np.all(np.isfinite(x))
    # Hermitian projections and unitary rotations: the stopping test bounds the true residual
    op.set_option(hw.OPT_COMPLEX_ARNOLDI, 1)
    x, it, res = op.gmres(b, max_iter=200, tol_pow=10)
    assert res < 1e-10
    assert relerr(op.matvec(x), b) < 1e-9
    assert relerr(x, xt) < 1e-8


@pytest.mark.gpu
def test_helmholtz_refuses_real_only_entry_points(gpu):
    hw = gpu
    op = helm_op(hw, 4096, 2, 6)
    x = cvec(3, op.N)
    with pytest.raises(hw.H2WError) as e:
        op.matvec(x, precision=hw.PREC_FP32)
    assert e.value.code == hw.ERR_ARG
    with pytest.raises(hw.H2WError) as e:
        op.gmres_ir(x.real)
    assert e.value.code == hw.ERR_ARG
    with pytest.raises(hw.H2WError) as e:
        op.autotune(nrhs=64)
    assert e.value.code == hw.ERR_ARG


# ------------------------------------------------------------- 2D Hankel ---
def hankel_op(hw, n, nlev, tol, form=0, seed=11):
    op = hw.H2Operator(2, form, hw.KERNEL_HANKEL, tol, nlev, device=0)
    op.set_points(synth.uniform_points(synth.config_seed(97, seed), n, 2))
    op.build_tree()
    op.assemble(hw.ASSEMBLE_NCA)
    return op


@pytest.mark.gpu
def test_hankel_entries_match_independent_values(gpu):
    """Column 0 of the 2D Hankel kernel matrix from the GPU's entries (dense
    product with e_0) against (-Y0 + i J0) / 4 from scipy, and the diagonal
    (1 + 15 ln N + Kii) / h^2 with Kii integrated from scipy's Bessel values
    (tests/golden/make_bessel.py)."""
    import os
    hw = gpu
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bessel_j0y0.npz"))
    pts = g["hankel_points"]
    n = len(pts)
    op = hw.H2Operator(2, 0, hw.KERNEL_HANKEL, 8, 2, device=0)
    op.set_points(pts)
    op.build_tree()
    e0 = np.zeros(n, dtype=np.complex128)
    e0[0] = 1.0
    col = op.dense_matvec(e0)
    ref = g["hankel_col0"]
    assert np.max(np.abs(col - ref) / np.abs(ref)) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_hankel_product_and_gmres(gpu, form):
    """2D Hankel on 16 384 random points, 3 levels, tol 1e-8: the compressed
    product against exact dense rows, complex linearity, and GMRES to 1e-10."""
    hw = gpu
    n = 16384
    op = hankel_op(hw, n, 3, 8, form)
    x = cvec(4, n)
    y = op.matvec(x)
    rows = np.arange(0, n, 257)[:64]
    yd = np.concatenate([op.dense_matvec(x, row0=int(r), nrows=1) for r in rows])
    assert relerr(y[rows], yd) < 1e-7
    x2 = cvec(5, n)
    a = -0.8 + 0.6j
    assert relerr(op.matvec(a * x + x2), a * y + op.matvec(x2)) < 1e-13
    # the reference's GMRES as written stops on its own estimate; with Hermitian
    # projections and unitary rotations the estimate bounds the true residual
    xs, it, res = op.gmres(y, max_iter=300, tol_pow=10)
    assert res < 1e-10 and it >= 1 and np.all(np.isfinite(xs))
    op.set_option(hw.OPT_COMPLEX_ARNOLDI, 1)
    xs, it2, res = op.gmres(y, max_iter=300, tol_pow=10)
    assert res < 1e-10 and it2 >= 1
    assert relerr(op.matvec(xs), y) < 1e-9
    assert relerr(xs, x) < 1e-6


@pytest.mark.gpu
def test_helmholtz_operator_file_round_trip(gpu, tmp_path):
    """An operator file of a complex operator (points and pivots) reopens to
    the same operator: the products agree bit for bit."""
    hw = gpu
    op = helm_op(hw, 6000, 2, 8)
    x = cvec(6, op.N)
    y = op.matvec(x)
    path = str(tmp_path / "helm.h2wop")
    op.save(path)
    op2 = hw.H2Operator.open(path)
    assert op2.complex and op2.storage_entries() == op.storage_entries()
    assert np.array_equal(op2.matvec(x), y)


@pytest.mark.gpu
def test_helmholtz_against_the_oracle(gpu):
    """Seeded random points outside the fixtures: the GPU product on the CPU
    oracle's pivots (the restatement, bit-exact with the reference's complex
    build) matches the oracle's product to 1e-13, and GMRES takes the
    oracle's iteration count +-1."""
    from oracle import Oracle
    hw = gpu
    n = 6000
    pts = synth.uniform_points(synth.config_seed(97, 21), n, 3)
    o = Oracle(3, 0, pts, 2, 8, hw.KERNEL_HELMHOLTZ)
    op = hw.H2Operator(3, 0, hw.KERNEL_HELMHOLTZ, 8, 2, device=0)
    op.set_points(pts)
    op.build_tree()
    for nm in ("far_check", "far_charge", "ver_check", "ver_charge"):
        op.import_list(nm, *o.csr(nm))
    op.assemble(hw.ASSEMBLE_IMPORT)
    assert op.storage_entries() == o.memory()
    x = cvec(7, n)
    assert relerr(op.matvec(x), o.matvec(x)) <= 1e-13
    b = o.dense_matvec(cvec(8, n))
    xs, it, res = op.gmres(b, max_iter=200, tol_pow=10)
    xo, ito, reso = o.gmres(b, max_iter=200, tol_pow=10)
    assert abs(it - ito) <= 1 and res < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_hankel_against_the_oracle(gpu, form):
    """2D Hankel on seeded random points against the CPU oracle (its own
    J0 / Y0 in long double; the reference's Hankel build needs Boost): the
    GPU's own pivots agree with the oracle's on most boxes, the product on the
    oracle's pivots matches the oracle's to 1e-13, GMRES takes its iteration
    count +-1."""
    from oracle import Oracle
    hw = gpu
    n = 4000
    pts = synth.uniform_points(synth.config_seed(97, 31 + form), n, 2)
    o = Oracle(2, form, pts, 3, 8, hw.KERNEL_HANKEL)
    names = ("far_check", "far_charge", "ver_check", "ver_charge") if form == 0 else ("far_check", "far_charge",
                                                                                      "sn_row", "sn_col")
    own = hw.H2Operator(2, form, hw.KERNEL_HANKEL, 8, 3, device=0)
    own.set_points(pts)
    own.build_tree()
    own.assemble(hw.ASSEMBLE_NCA)
    agree = total = 0
    for nm in names:
        p, v = own.get_list(nm)
        q, w = o.csr(nm)
        for i in range(len(q) - 1):
            total += 1
            agree += int(np.array_equal(v[p[i]:p[i + 1]], w[q[i]:q[i + 1]]))
    assert agree >= 0.9 * total, (agree, total)
    assert abs(own.storage_entries() - o.memory()) <= 0.01 * o.memory()
    op = hw.H2Operator(2, form, hw.KERNEL_HANKEL, 8, 3, device=0)
    op.set_points(pts)
    op.build_tree()
    for nm in names:
        op.import_list(nm, *o.csr(nm))
    op.assemble(hw.ASSEMBLE_IMPORT)
    assert op.storage_entries() == o.memory()
    x = cvec(9, n)
    assert relerr(op.matvec(x), o.matvec(x)) <= 1e-13
    b = o.dense_matvec(cvec(10, n))
    xs, it, res = op.gmres(b, max_iter=200, tol_pow=10)
    xo, ito, reso = o.gmres(b, max_iter=200, tol_pow=10)
    assert abs(it - ito) <= 1 and res < 1e-10
