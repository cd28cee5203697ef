"""The reference's GMRES (restated, oracle/gmres_ref.hpp) drives the GPU
operator through the C++ adapter (include/h2w_adapter.hpp), compiled and run
as a reference driver would be: iterations within +-1 and solution error
within 10x of the CPU oracle's GMRES on the same problem."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from h2weak_gb300 import synth


@pytest.mark.gpu
@pytest.mark.parametrize("case", [(2, 0, 64, 4, 10, 0), (1, 0, 8192, 7, 10, 1), (3, 1, 20, 3, 8, 1)])
def test_reference_gmres_through_the_adapter(gpu, tmp_path, case):
    hw = gpu
    from oracle import Oracle
    dim, form, n, nl, tol, ch = case
    exe = str(tmp_path / "adapter_gmres")
    lib = os.path.join(ROOT, "h2weak_gb300", "_lib")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "oracle", "eigen_shim"), "-I", os.path.join(ROOT, "oracle"),
                        os.path.join(ROOT, "tests", "adapter_gmres.cpp"), "-L", lib, "-lh2w", "-Wl,-rpath," + lib,
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    N = n ** dim
    xt = synth.normal(synth.config_seed(76, dim), N)
    xf = str(tmp_path / "xt.bin")
    xt.tofile(xf)
    r = subprocess.run([exe, str(dim), str(form), str(n), str(nl), str(tol), str(ch), "10", xf], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    it, res, err, NN = r.stdout.split()
    it, res, err = int(it), float(res), float(err)
    assert int(NN) == N and res < 1e-10
    h = hw.H2Operator(dim, form, ch, tol, nl, device=-1)
    h.gen_grid(n)
    pts = h.points()
    o = Oracle(dim, form, pts, nl, tol, ch, N, 2 * N if dim == 1 else N)
    b = o.dense_matvec(xt)
    xo, ito, _ = o.gmres(b, max_iter=500, tol_pow=10)
    err_o = np.linalg.norm(xo - xt) / np.linalg.norm(xt)
    assert abs(it - ito) <= 1, (it, ito)
    assert err <= 10 * err_o + 1e-12, (err, err_o)
