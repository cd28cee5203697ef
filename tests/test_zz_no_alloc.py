"""h2w_matvec_static, the matvec entry point that allocates nothing (its
workspace is a fixed device array inside the library), called through the
C ABI and checked against h2w_matvec on the same operator and inputs, two
calls in a row per precision and per launch form. Also: no device memory is
taken by a call after the first, host pointers and a missing FP32 operator
copy are refused, an operator whose workspace exceeds the array is refused,
and a grid-barrier wait that runs out is reported by the call that ran it.
Kept in a file of its own that runs last and also runs alone in a fresh
process."""
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


def _operator(hw, n=64):
    op = hw.H2Operator(2, hw.FORM_NESTED, 0, 10, 4, device=0)
    op.gen_grid(n)
    op.build_tree()
    op.assemble()
    return op


@pytest.mark.gpu
@pytest.mark.parametrize("coop", [1, 0])
def test_static_workspace_matvec_matches_matvec(gpu, coop):
    import torch
    hw = gpu
    f = _entry(hw)
    op = _operator(hw)
    op.set_option(hw.OPT_COOP, coop)
    N = op.N
    x0 = torch.zeros(N, dtype=torch.float64, device="cuda")
    y0 = torch.empty_like(x0)
    # FP32 before the FP32 operator copy exists: refused, nothing launched
    assert f(op.h, P(x0.data_ptr()), P(y0.data_ptr()), hw.PREC_FP32, None) == hw.ERR_STATE
    # the FP32 operator copy comes from one call of the allocating entry point
    op.matvec(np.ones(N), precision=hw.PREC_FP32)
    for prec, tol in ((hw.PREC_FP64, 1e-13), (hw.PREC_FP32, 1e-6)):
        for call in range(2):
            x = torch.from_numpy(synth.normal(synth.config_seed(90 + prec, call), N)).cuda()
            y_static = torch.full_like(x, np.nan)
            y_ref = torch.empty_like(x)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            rc = f(op.h, P(x.data_ptr()), P(y_static.data_ptr()), prec, None)
            assert rc == 0, hw.lib().h2w_last_error(op.h)
            torch.cuda.synchronize()
            if call == 1:  # after the set-up call: no device memory taken
                assert torch.cuda.mem_get_info()[0] == free0
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


@pytest.mark.gpu
def test_static_workspace_matvec_refuses_host_pointers(gpu):
    import torch
    hw = gpu
    f = _entry(hw)
    op = _operator(hw, 32)
    xh = np.ones(op.N)
    yh = np.empty(op.N)
    yd = torch.empty(op.N, dtype=torch.float64, device="cuda")
    xd = torch.ones(op.N, dtype=torch.float64, device="cuda")
    assert f(op.h, P(xh.ctypes.data), P(yd.data_ptr()), hw.PREC_FP64, None) == hw.ERR_ARG
    assert f(op.h, P(xd.data_ptr()), P(yh.ctypes.data), hw.PREC_FP64, None) == hw.ERR_ARG
    assert f(op.h, P(xd.data_ptr()), P(yd.data_ptr()), hw.PREC_FP64, None) == 0


@pytest.mark.gpu
def test_static_workspace_matvec_reports_barrier_timeout(gpu):
    """A grid-barrier wait limited to one poll runs out (the kernel finishes
    with an invalid product): the call itself returns H2W_ERR_CUDA, and the
    next call with the ordinary limit is correct again."""
    import torch
    hw = gpu
    f = _entry(hw)
    op = _operator(hw)
    x = torch.from_numpy(synth.normal(synth.config_seed(97), op.N)).cuda()
    y = torch.empty_like(x)
    y_ref = torch.empty_like(x)
    op.set_option(hw.OPT_SPIN_LIMIT, 1)
    assert f(op.h, P(x.data_ptr()), P(y.data_ptr()), hw.PREC_FP64, None) == hw.ERR_CUDA
    assert b"grid-barrier" in hw.lib().h2w_last_error(op.h)
    op.set_option(hw.OPT_SPIN_LIMIT, 0)
    assert f(op.h, P(x.data_ptr()), P(y.data_ptr()), hw.PREC_FP64, None) == 0
    op.matvec_device(x.data_ptr(), y_ref.data_ptr(), precision=hw.PREC_FP64)
    torch.cuda.synchronize()
    a, b = y.cpu().numpy(), y_ref.cpu().numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-13


@pytest.mark.gpu
def test_static_workspace_matvec_refuses_oversized_operator(gpu):
    """An operator whose workspace (at least N doubles) exceeds the 2^21
    doubles of the array: refused with H2W_ERR_ARG before any launch."""
    import torch
    hw = gpu
    f = _entry(hw)
    n = (1 << 21) + 4096
    op = hw.H2Operator(1, hw.FORM_NESTED, 1, 6, 15, device=0)
    op.gen_grid(n)
    op.build_tree()
    op.assemble()
    x = torch.zeros(op.N, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    assert f(op.h, P(x.data_ptr()), P(y.data_ptr()), hw.PREC_FP64, None) == hw.ERR_ARG
    assert b"exceeds" in hw.lib().h2w_last_error(op.h)
