"""The NCA for large blocks (groups of CTAs of one cooperative launch)
against the one-CTA-per-block NCA on the same problem: the same pivots in
every list (an IEEE-exact kernel, so entries and residuals are bitwise
equal; the stopping test's sums are tree reductions in both, a near-tie could
differ in the last pivot), hence the same storage count and product."""
import os

import numpy as np
import pytest

from h2weak_gb300 import synth


def _lists(op, names):
    return {n: op.get_list(n) for n in names}


@pytest.mark.gpu
@pytest.mark.parametrize("spec", [(2, 0, 1, 10, 128, 4), (2, 1, 1, 10, 128, 4)])
def test_group_nca_matches_single_cta(gpu, spec):
    hw = gpu
    from h2weak_gb300 import learned
    dim, form = spec[0], spec[1]
    names = ["far_check", "far_charge", "ver_check", "ver_charge"] if form == 0 else ["far_check", "far_charge", "sn_row", "sn_col"]
    ops = {}
    try:
        for mode in ("1", "0"):
            os.environ["H2W_NCA_BIG"] = mode
            op = learned.make_problem(hw, spec)
            op.assemble(hw.ASSEMBLE_NCA)
            ops[mode] = op
    finally:
        os.environ.pop("H2W_NCA_BIG", None)
    a, b = _lists(ops["1"], names), _lists(ops["0"], names)
    same = 0
    total = 0
    for n in names:
        pa, va = a[n]
        pb, vb = b[n]
        for i in range(len(pa) - 1):
            total += 1
            same += int(np.array_equal(va[pa[i]:pa[i + 1]], vb[pb[i]:pb[i + 1]]))
    assert same >= 0.99 * total, (same, total)
    sa, sb = ops["1"].storage_entries(), ops["0"].storage_entries()
    assert abs(sa - sb) <= 1e-3 * sb
    x = synth.normal(synth.config_seed(91, 0), ops["1"].N)
    ya, yb = ops["1"].matvec(x), ops["0"].matvec(x)
    yd = ops["0"].dense_matvec(x, 0, 256)
    ea = np.linalg.norm(ya[:256] - yd) / np.linalg.norm(yd)
    eb = np.linalg.norm(yb[:256] - yd) / np.linalg.norm(yd)
    assert ea <= 10 * eb + 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("spec", [(2, 0, 0, 10, 128, 4), (3, 0, 1, 10, -30000, 3)])
def test_double_fp32_group_search_matches_fp64(gpu, spec):
    """Kernels built on log: the group search in double-FP32 arithmetic (the
    default for them) against the FP64 search on the same problem: pivot lists
    equal on nearly every box, storage within 0.5 %, the same accuracy against
    exact dense rows."""
    hw = gpu
    from h2weak_gb300 import learned
    names = ["far_check", "far_charge", "ver_check", "ver_charge"]
    ops = {}
    for df in (1, 0):
        op = learned.make_problem(hw, spec)
        op.set_option(hw.OPT_NCA_DF, df)
        op.assemble(hw.ASSEMBLE_NCA)
        ops[df] = op
    a, b = _lists(ops[1], names), _lists(ops[0], names)
    same = total = 0
    for n in names:
        pa, va = a[n]
        pb, vb = b[n]
        for i in range(len(pa) - 1):
            total += 1
            same += int(np.array_equal(va[pa[i]:pa[i + 1]], vb[pb[i]:pb[i + 1]]))
    assert same >= 0.95 * total, (same, total)
    sa, sb = ops[1].storage_entries(), ops[0].storage_entries()
    assert abs(sa - sb) <= 5e-3 * sb
    x = synth.normal(synth.config_seed(92, 0), ops[1].N)
    yd = ops[0].dense_matvec(x, 0, 256)
    ea = np.linalg.norm(ops[1].matvec(x)[:256] - yd) / np.linalg.norm(yd)
    eb = np.linalg.norm(ops[0].matvec(x)[:256] - yd) / np.linalg.norm(yd)
    assert ea <= 10 * eb + 1e-13, (ea, eb)
