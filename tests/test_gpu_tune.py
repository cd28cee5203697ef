"""Target-stream re-cuts and the autotuner: any column cap of the
multi-vector stream and any row split of the single-vector stream give the
same products (to atomic-accumulation rounding); the autotuner keeps one of
its candidates and the products stay correct afterwards."""
import numpy as np
import pytest

from h2weak_gb300 import synth
from test_gpu_oracle import setup

CASES = [(2, 0, 64, None, 4, 10, 0), (3, 1, 24, None, 3, 8, 1)]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_recut_streams_same_products(gpu, case):
    hw = gpu
    op, _ = setup(hw, case)
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    X = np.stack([synth.normal(synth.config_seed(85, c), N) for c in range(20)], axis=1)
    Y0 = op.matvec(X)
    y0 = op.matvec(X[:, 0])
    assert op.get_option(hw.OPT_MULTI_XW) == 1024
    st0 = op.plan_stats()
    # stored panels keep their columns at 4-row strides: the plan reads at most the stored entries
    assert 0 < st0["entries"] <= op.storage_entries()
    for cap in (256, 512, 2048, 32):
        op.set_option(hw.OPT_MULTI_XW, cap)
        assert op.get_option(hw.OPT_MULTI_XW) == cap
        st = op.plan_stats()
        # a re-cut moves entries between targets, never adds or drops any
        assert st["entries"] == st0["entries"]
        assert st["entries"] <= st["multiplied"] <= st["tile_span"]
        if cap == 32:
            assert st["atomic_targets"] > 0 and st["targets"] > st0["targets"]
        Y = op.matvec(X)
        for c in range(20):
            assert rel(Y[:, c], Y0[:, c]) < 1e-13, (cap, c)
        Yf = op.matvec(X, precision=hw.PREC_FP32)
        assert rel(Yf[:, 5], Y0[:, 5]) < 1e-5
    for rs in (4096, 65536):
        op.set_option(hw.OPT_ROW_SPLIT, rs)
        assert rel(op.matvec(X[:, 0]), y0) < 1e-13
        assert rel(op.matvec(X[:, 0], precision=hw.PREC_FP32), y0) < 1e-5
    with pytest.raises(hw.H2WError):
        op.set_option(hw.OPT_MULTI_XW, 4096 * 4)
    with pytest.raises(hw.H2WError):
        op.set_option(hw.OPT_MULTI_XW, 250)


@pytest.mark.gpu
def test_autotune_keeps_a_candidate(gpu):
    hw = gpu
    op, _ = setup(hw, CASES[0])
    op.assemble(hw.ASSEMBLE_NCA)
    N = op.N
    X = np.stack([synth.normal(synth.config_seed(86, c), N) for c in range(64)], axis=1)
    Y0 = op.matvec(X)
    cap, ms = op.autotune(nrhs=64, precision=hw.PREC_DF64, reps=2)
    assert cap in (256, 512, 1024, 2048) and ms > 0
    cap, ms = op.autotune(nrhs=64, precision=hw.TUNE_IR_MIX, reps=1)
    assert cap in (256, 512, 1024, 2048) and ms > 0
    assert op.get_option(hw.OPT_MULTI_XW) == cap
    # the FP32 product's form is a candidate too; either gives the product
    assert op.get_option(hw.OPT_PRODUCER_WARP) in (0, 1)
    Yf = op.matvec(X, precision=hw.PREC_FP32)
    assert max(rel(Yf[:, c], Y0[:, c]) for c in range(64)) < 1e-5
    Y = op.matvec(X, precision=hw.PREC_DF64)
    assert max(rel(Y[:, c], Y0[:, c]) for c in range(64)) < 1e-12
    rs, ms1 = op.autotune(nrhs=1, precision=hw.PREC_FP32, reps=3)
    assert rs in (4096, 8192, 16384, 32768, 65536) and ms1 > 0
    assert op.get_option(hw.OPT_ROW_SPLIT) == rs
    assert rel(op.matvec(X[:, 7]), Y0[:, 7]) < 1e-13
    # the solvers run on the re-cut streams
    Xs, it, res = op.gmres_batch(Y0[:, :8], max_iter=200, tol_pow=10)
    assert np.all(res < 1e-10)
