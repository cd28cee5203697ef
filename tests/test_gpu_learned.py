"""Learned NCA proposals: the network's GPU forward and gradient kernels
against the CPU oracle; training on recorded NCA data lowers the loss; the
learned assembly meets the NCA tolerance (matvec error against the dense
product on sampled rows as plain NCA's) and a trained network gets more
blocks accepted than an untrained one."""
import ctypes
import time

import numpy as np
import pytest

from h2weak_gb300 import synth


def _dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
def test_mlp_kernels_match_oracle(gpu):
    import torch
    import mlp_ref
    hw = gpu
    L = hw.lib()
    rng = np.random.default_rng(5)
    n = 257  # a partial last tile
    X = rng.normal(size=(n, 16)).astype(np.float32)
    y = (rng.random(n) < 0.2).astype(np.uint8)
    p = np.concatenate([rng.normal(0, 0.2, s) for _, s in mlp_ref.SIZES]).astype(np.float32)
    assert len(p) == L.h2w_mlp_nparam()
    pd, Xd, yd = _dev(p, torch), _dev(X, torch), _dev(y, torch)
    z = torch.empty(n, dtype=torch.float32, device="cuda")
    g = torch.empty_like(pd)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    assert L.h2w_mlp_forward(ctypes.c_void_p(pd.data_ptr()), ctypes.c_void_p(Xd.data_ptr()), n,
                             ctypes.c_void_p(z.data_ptr()), None) == 0
    assert L.h2w_mlp_grad(ctypes.c_void_p(pd.data_ptr()), ctypes.c_void_p(Xd.data_ptr()),
                          ctypes.c_void_p(yd.data_ptr()), n, 3.0, ctypes.c_void_p(g.data_ptr()),
                          ctypes.c_void_p(loss.data_ptr()), None) == 0
    torch.cuda.synchronize()
    zo, _ = mlp_ref.forward(p, X)
    lo, go = mlp_ref.loss_grad(p, X, y, 3.0)
    assert np.max(np.abs(z.cpu().numpy() - zo)) <= 1e-4 * max(1.0, np.max(np.abs(zo)))
    assert abs(float(loss.item()) - lo) <= 1e-4 * abs(lo)
    gg = g.cpu().numpy()
    o = 0
    for name, size in mlp_ref.SIZES:
        a, b = gg[o:o + size], go[o:o + size]
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b) + 1e-9, name
        o += size


def _dense_rows_err(op, x, rows=256):
    y = op.matvec(x)
    yd = op.dense_matvec(x, 0, rows)
    return np.linalg.norm(y[:rows] - yd) / np.linalg.norm(yd)


@pytest.mark.gpu
def test_train_and_learned_assembly(gpu):
    import h2weak_gb300 as hw
    from h2weak_gb300 import learned
    specs = [(2, 0, 0, 10, 64, 3), (2, 0, 1, 10, 64, 3), (2, 0, 1, 8, -6000, 3), (3, 0, 0, 8, 16, 2)]
    X, y = learned.collect(specs)
    assert len(y) > 10000 and 0 < y.sum() < len(y)
    p0 = learned.init_params(1)
    params, losses = learned.train(X, y, epochs=6, batch=32768, lr=3e-3, params=p0)
    assert losses[-1] < 0.8 * losses[0]
    calib = learned.calibrate(params, X, y)
    assert 0.05 < calib < 20
    # a problem outside the training set
    spec = (2, 0, 0, 10, 96, 3)
    x = synth.normal(synth.config_seed(89, 0), 96 * 96)
    plain = learned.make_problem(hw, spec)
    t0 = time.time()
    plain.assemble(hw.ASSEMBLE_NCA)
    t_plain = time.time() - t0
    e_plain = _dense_rows_err(plain, x)
    stats = {}
    for name, prm, cal in (("trained", params, calib), ("untrained", p0, 1.0)):
        op = learned.make_problem(hw, spec)
        op.learn_set_model(prm, 2.0 * cal, 4)  # oversampled proposals, trimmed by the small ACA
        t0 = time.time()
        op.assemble(hw.ASSEMBLE_LEARNED)
        t = time.time() - t0
        print(name, op.learn_detail())
        blocks, acc = op.learn_stats()
        e = _dense_rows_err(op, x)
        assert e <= 10 * e_plain + 1e-12, (name, e, e_plain)
        # accepted proposals keep the NCA's tolerance at about the plain ranks
        assert op.storage_entries() <= 1.05 * plain.storage_entries(), (name, op.storage_entries(),
                                                                        plain.storage_entries())
        stats[name] = (blocks, acc, t, e)
    print("plain %.3fs err %.2e; " % (t_plain, e_plain) + "; ".join(
        "%s: %d/%d accepted, %.3fs, err %.2e" % (k, v[1], v[0], v[2], v[3]) for k, v in stats.items()))
    assert stats["trained"][1] > stats["untrained"][1]
    assert stats["trained"][1] >= 0.5 * stats["trained"][0]
