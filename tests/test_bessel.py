"""The library's FP64 J0 and Y0 (h2weak_gb300/csrc/bessel.cuh, used by the 2D
Hankel kernel) against scipy's (Cephes) on arguments across the power-series,
double-double and asymptotic regimes; host build with g++."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def j0y0(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("bessel") / "libbessel.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", os.path.join(HERE, "bessel_batch.cpp"), "-o", out],
                   check=True)
    lib = ctypes.CDLL(out)
    lib.j0y0_batch.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]

    def f(x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        j, y = np.empty_like(x), np.empty_like(x)
        lib.j0y0_batch(x.ctypes.data, x.size, j.ctypes.data, y.ctypes.data)
        return j, y
    return f


def test_j0_y0_match_independent_values(j0y0):
    g = np.load(os.path.join(HERE, "golden", "bessel_j0y0.npz"))
    x = g["x"]
    j, y = j0y0(x)
    # error relative to max(|f|, envelope sqrt(2 / (pi x))): absolute near the zeros
    env = np.sqrt(2.0 / (np.pi * np.maximum(x, 1.0)))
    ej = np.abs(j - g["j0"]) / np.maximum(np.abs(g["j0"]), env)
    ey = np.abs(y - g["y0"]) / np.maximum(np.abs(g["y0"]), env)
    assert ej.max() < 1e-14, ej.max()
    assert ey.max() < 1e-14, ey.max()


def test_library_and_oracle_bessel_agree(j0y0):
    """The oracle's own J0 / Y0 (a long-double power series, for its 2D Hankel
    entries) and the library's agree, pair distances in (0, 2.83]: the 2D
    Hankel entries of the oracle's column 0 against (-Y0 + i J0) / 4 from the
    library's functions."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
    sys.path.insert(0, os.path.join(HERE, ".."))
    from oracle import Oracle
    from h2weak_gb300 import synth
    pts = synth.uniform_points(synth.config_seed(98, 3), 2000, 2)
    o = Oracle(2, 0, pts, 2, 8, 10, assemble=False)
    col = o.entries(np.arange(1, len(pts)), [0])[:, 0]
    R = np.sqrt(((pts[1:] - pts[0]) ** 2).sum(axis=1))
    j, y = j0y0(R)
    lib = (-y + 1j * j) / 4.0
    assert np.max(np.abs(col - lib) / np.abs(lib)) < 1e-14
