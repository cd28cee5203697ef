"""The CPU oracle reproduces the storage known-answer values the reference
publishes ({1D,2D,3D}/results/*.txt, nested, semi-nested and non-nested forms: Storage (in GB) = memory*8e-9 and
Compression ratio = memory/N^2, printed with 6 significant digits)."""
import pytest

import h2weak_gb300 as hw

CASES = [
    # dim, form, n_param, nLevels, tol, choice, published storage GB, published ratio
    (1, 0, 250000, 12, 12, 1, "0.658597", "0.00131719"),   # 1D/results/nhodlr.txt:25-27
    (1, 1, 250000, 12, 12, 1, "1.61", "0.00322"),          # 1D/results/sn_hodlr.txt:25-27
    (3, 1, 35, 3, 7, 0, "3.02412", "0.205637"),            # 3D/results/sn_hodlr.txt:25-27 (tol 1e-7, 3D/README.md:2)
    (2, 2, 300, 4, 12, 1, "4.17922", "0.0644941"),         # 2D/results/hodlr.txt:25-27 (non-nested H*)
    (3, 2, 35, 3, 7, 0, "4.39326", "0.298737"),            # 3D/results/hodlr.txt:25-27 (non-nested H*)
]


def g6(x):
    return "%g" % x


@pytest.mark.parametrize("case", CASES)
def test_oracle_reproduces_published_storage(case):
    from oracle import Oracle
    dim, form, n, nl, tol, ch, gb, ratio = case
    op = hw.H2Operator(dim, form, ch, tol, nl, device=-1)
    op.gen_grid(n)
    pts = op.points()
    N = len(pts)
    o = Oracle(dim, form, pts, nl, tol, ch, N, 2 * N if dim == 1 else N)
    mem = o.memory()
    assert g6(mem * 8 * 10.0 ** -9) == gb
    assert g6(mem / (1.0 * N * N)) == ratio
