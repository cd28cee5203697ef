import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


# Fixtures of reference builds that the library does not provide (the complex
# kernels in the non-nested H* form, which h2w_create refuses): only the
# oracle's tests use them.
ORACLE_ONLY_GOLDEN = ("g2d_nn_hankel", "g3d_nn_helm")


def golden_names(oracle=False):
    names = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and f.startswith("g"))
    return names if oracle else [n for n in names if n not in ORACLE_ONLY_GOLDEN]


def load_golden(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    s = d["spec"]
    d["dim"], d["form"], d["n_param"], d["nlevels"], d["leaf"], d["tol_pow"], d["choice"], d["gtol"], d["N"] = \
        (int(v) for v in s)
    return d


def csr_split(ptr, val):
    return [val[ptr[i]:ptr[i + 1]] for i in range(len(ptr) - 1)]


@pytest.fixture(scope="session")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import h2weak_gb300 as hw
    hw.build()
    return hw
