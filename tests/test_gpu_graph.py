"""CUDA-graph GMRES: the Arnoldi steps captured once as the body of a
conditional while node give the host-driven loop's results (same kernels,
same order): bitwise for the single-vector FP64 and mixed solvers, converged
or stopped at max_iter, and to rounding for the batched solvers; and the
capture is really used."""
import numpy as np
import pytest

from h2weak_gb300 import synth
from test_gpu_oracle import setup

CASE2 = (2, 0, 64, None, 4, 10, 0)
CASE3 = (3, 1, 24, None, 3, 8, 1)


def _op(hw, case):
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    return op


@pytest.mark.gpu
@pytest.mark.parametrize("case", [CASE2, CASE3])
def test_graph_gmres_bitwise(gpu, case):
    hw = gpu
    op = _op(hw, case)
    N = op.N
    b = op.dense_matvec(synth.normal(synth.config_seed(80, 0), N))
    op.set_option(hw.OPT_GRAPH, 1)
    xg, itg, rg = op.gmres(b, max_iter=200, tol_pow=10)
    assert op.get_option(hw.OPT_GRAPH) == 1  # the capture succeeded and was used
    op.set_option(hw.OPT_GRAPH, 0)
    xh, ith, rh = op.gmres(b, max_iter=200, tol_pow=10)
    assert itg == ith and rg == rh
    assert np.array_equal(xg, xh)
    # stopped at max_iter (not converged): same partial solution both ways
    op.set_option(hw.OPT_GRAPH, 1)
    xg3, itg3, _ = op.gmres(b, max_iter=3, tol_pow=14)
    op.set_option(hw.OPT_GRAPH, 0)
    xh3, ith3, _ = op.gmres(b, max_iter=3, tol_pow=14)
    assert itg3 == ith3 == 3
    assert np.array_equal(xg3, xh3)


@pytest.mark.gpu
def test_graph_gmres_ir_bitwise(gpu):
    hw = gpu
    op = _op(hw, CASE2)
    b = op.dense_matvec(synth.normal(synth.config_seed(81, 0), op.N))
    op.set_option(hw.OPT_GRAPH, 1)
    xg, og, ig, rg = op.gmres_ir(b, max_outer=20, inner_iter=100, tol_pow=10)
    assert op.get_option(hw.OPT_GRAPH) == 1
    op.set_option(hw.OPT_GRAPH, 0)
    xh, oh, ih, rh = op.gmres_ir(b, max_outer=20, inner_iter=100, tol_pow=10)
    assert (og, ig, rg) == (oh, ih, rh)
    assert np.array_equal(xg, xh)
    assert rg < 1e-10


@pytest.mark.gpu
def test_graph_gmres_batch(gpu):
    """Batched solvers, graph against host loop. The multi-vector product
    accumulates column-split targets with atomics, so the two runs agree to
    rounding (not bitwise): same iteration counts (+-1), both converged, the
    solutions within 1e-9 of each other."""
    hw = gpu
    op = _op(hw, CASE3)
    N = op.N
    XT = np.stack([synth.normal(synth.config_seed(82, c), N) for c in range(6)], axis=1)
    B = op.matvec(XT)
    op.set_option(hw.OPT_GRAPH, 1)
    Xg, itg, rg = op.gmres_batch(B, max_iter=200, tol_pow=10)
    assert op.get_option(hw.OPT_GRAPH) == 1
    op.set_option(hw.OPT_GRAPH, 0)
    Xh, ith, rh = op.gmres_batch(B, max_iter=200, tol_pow=10)
    assert np.all(np.abs(itg - ith) <= 1)
    assert np.all(rg < 1e-10) and np.all(rh < 1e-10)
    for c in range(6):
        assert np.linalg.norm(Xg[:, c] - Xh[:, c]) / np.linalg.norm(Xh[:, c]) < 1e-9
    op.set_option(hw.OPT_GRAPH, 1)
    Xg, og, ig, rg = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=10)
    op.set_option(hw.OPT_GRAPH, 0)
    Xh, oh, ih, rh = op.gmres_ir_batch(B, max_outer=20, inner_iter=100, tol_pow=10)
    assert og == oh and abs(ig - ih) <= og
    assert np.all(rg < 1e-10) and np.all(rh < 1e-10)
    for c in range(6):
        assert np.linalg.norm(Xg[:, c] - Xh[:, c]) / np.linalg.norm(Xh[:, c]) < 1e-9


@pytest.mark.gpu
def test_graph_with_per_phase_launches(gpu):
    """The captured step also works with one launch per matvec phase."""
    hw = gpu
    op = _op(hw, CASE2)
    b = op.dense_matvec(synth.normal(synth.config_seed(83, 0), op.N))
    x1, it1, _ = op.gmres(b, max_iter=200, tol_pow=10)
    op.set_option(hw.OPT_COOP, 0)
    op.set_option(hw.OPT_GRAPH, 1)
    x2, it2, _ = op.gmres(b, max_iter=200, tol_pow=10)
    assert op.get_option(hw.OPT_GRAPH) == 1
    assert abs(it1 - it2) <= 1
    assert np.linalg.norm(x1 - x2) / np.linalg.norm(x1) < 1e-9
