"""h2w_matvec_static, the matvec entry point that allocates nothing (its
workspace is a fixed device array inside the library), called through the
C ABI and checked against h2w_matvec on the same operator and inputs, two
calls in a row per precision. Kept in a file of its own that runs last and
also runs alone in a fresh process."""
import ctypes

import numpy as np
import pytest

from h2weak_gb300 import synth

P, I = ctypes.c_void_p, ctypes.c_int


def _entry(hw):
    f = hw.lib().h2w_matvec_static
    f.argtypes = [P, P, P, I, P]
    f.restype = I
    return f


@pytest.mark.gpu
def test_static_workspace_matvec_matches_matvec(gpu):
    import torch
    hw = gpu
    f = _entry(hw)
    op = hw.H2Operator(2, hw.FORM_NESTED, 0, 10, 4, device=0)
    op.gen_grid(64)
    op.build_tree()
    op.assemble()
    N = op.N
    # the FP32 operator copy comes from one call of the allocating entry point
    op.matvec(np.ones(N), precision=hw.PREC_FP32)
    for prec, tol in ((hw.PREC_FP64, 1e-13), (hw.PREC_FP32, 1e-6)):
        for call in range(2):
            x = torch.from_numpy(synth.normal(synth.config_seed(90 + prec, call), N)).cuda()
            y_static = torch.full_like(x, np.nan)
            y_ref = torch.empty_like(x)
            rc = f(op.h, P(x.data_ptr()), P(y_static.data_ptr()), prec, None)
            assert rc == 0, hw.lib().h2w_last_error(op.h)
            op.matvec_device(x.data_ptr(), y_ref.data_ptr(), precision=prec)
            torch.cuda.synchronize()
            a, b = y_static.cpu().numpy(), y_ref.cpu().numpy()
            assert np.all(np.isfinite(a))
            assert np.linalg.norm(a - b) / np.linalg.norm(b) <= tol, (prec, call)


@pytest.mark.gpu
def test_static_workspace_matvec_refuses_without_operator(gpu):
    hw = gpu
    f = _entry(hw)
    op = hw.H2Operator(2, hw.FORM_NESTED, 0, 10, 4, device=0)
    op.gen_grid(16)
    op.build_tree()
    rc = f(op.h, P(0), P(0), hw.PREC_FP64, None)
    assert rc == hw.ERR_STATE
