"""Generate tests/golden/bessel_j0y0.npz: J0 and Y0 from scipy.special (an
independent implementation, the Cephes library) on arguments spanning the
library's three evaluation regimes (power series, double-double series,
asymptotic expansion), and the entries of the 2D Hankel kernel (choice 10)
for a small seeded point set: column 0 of K, with the diagonal
(1 + 15 ln N + Kii) / h^2 and Kii the 16 x 16 Gauss-Legendre integral of
i H0^(1)(R) / 4 over [0, h/2]^2 times 4 (2D/codes/kernel.hpp:101-144,
2D/codes/integral2d.hpp:16-90). Needs scipy (this container); the committed
.npz is what the tests read.

    python tests/golden/make_bessel.py
"""
import os
import sys

import numpy as np
import scipy.special as sp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
from h2weak_gb300 import synth  # noqa: E402


def main():
    x = np.concatenate([np.logspace(-8, 0, 200), np.linspace(1.0, 40.0, 1200), np.linspace(3.9, 4.1, 41),
                        np.linspace(23.9, 24.1, 41)])
    n = 300
    pts = synth.uniform_points(synth.config_seed(98, 0), n, 2)
    R = np.sqrt((pts[:, 0] - pts[0, 0]) ** 2 + (pts[:, 1] - pts[0, 1]) ** 2)
    with np.errstate(invalid="ignore", divide="ignore"):  # R = 0 at the diagonal, replaced below
        col = (-sp.y0(R) + 1j * sp.j0(R)) / 4.0
    h = 1.0 / np.sqrt(n)
    gx, gw = np.polynomial.legendre.leggauss(16)
    c = 0.25 * h
    tx = c * gx + c
    TX, TY = np.meshgrid(tx, tx, indexing="ij")
    RR = np.sqrt(TX ** 2 + TY ** 2)
    f = (-sp.y0(RR) + 1j * sp.j0(RR)) / 4.0
    kii = (np.outer(gw, gw) * f).sum() * c * c * 4
    col[0] = (1.0 + 15 * np.log(n) + kii) / h ** 2
    np.savez_compressed(os.path.join(HERE, "bessel_j0y0.npz"), x=x, j0=sp.j0(x), y0=sp.y0(x), hankel_points=pts,
                        hankel_col0=col, hankel_kii=kii)


if __name__ == "__main__":
    main()
