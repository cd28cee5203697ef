"""The C++ adapter (include/h2w_adapter.hpp) compiles against a vector type
with the Eigen API subset the reference uses."""
import os
import subprocess

from conftest import ROOT


def test_adapter_compiles(tmp_path):
    src = tmp_path / "use_adapter.cpp"
    src.write_text('#include <Eigen/Dense>\n#include "h2w_adapter.hpp"\n'
                   "template class h2w_initialisation<Eigen::VectorXd>;\n"
                   "int main() { return 0; }\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "oracle", "eigen_shim"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
