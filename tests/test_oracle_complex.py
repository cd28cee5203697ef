"""The CPU oracle's complex kernels on their own: the 3D Helmholtz kernel
(bit-exact with the reference's USE_Helm build through the golden fixtures,
tests/test_oracle_golden.py) and the 2D Hankel kernel, whose reference build
needs Boost and cannot be built here: its entries against scipy's J0 / Y0
(tests/golden/bessel_j0y0.npz), its compressed product against its dense
product, and its GMRES."""
import os

import numpy as np
import pytest

from oracle import Oracle
from h2weak_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))


def test_hankel_entries_match_independent_values():
    g = np.load(os.path.join(HERE, "golden", "bessel_j0y0.npz"))
    pts = g["hankel_points"]
    o = Oracle(2, 0, pts, 2, 8, 10, assemble=False)
    col = o.entries(np.arange(len(pts)), [0])[:, 0]
    ref = g["hankel_col0"]
    assert np.max(np.abs(col - ref) / np.abs(ref)) < 1e-14


@pytest.mark.parametrize("form", [0, 1])
def test_hankel_operator_and_gmres(form):
    n = 3000
    pts = synth.uniform_points(synth.config_seed(99, form), n, 2)
    o = Oracle(2, form, pts, 3, 8, 10)
    x = synth.normal(synth.config_seed(99, 10), n) + 1j * synth.normal(synth.config_seed(99, 11), n)
    y = o.matvec(x)
    yd = o.dense_matvec(x)
    assert np.linalg.norm(y - yd) / np.linalg.norm(yd) < 1e-7
    xs, it, res = o.gmres(yd, max_iter=200, tol_pow=10)
    assert res < 1e-10 and 1 <= it <= 200


def test_complex_refusals():
    pts = synth.uniform_points(synth.config_seed(99, 20), 100, 3)
    with pytest.raises(ValueError):
        Oracle(3, 0, pts, 2, 8, 10)  # the Hankel kernel is 2D
    with pytest.raises(ValueError):
        Oracle(2, 0, pts[:, :2], 2, 8, 2)  # the Helmholtz kernel is 3D
