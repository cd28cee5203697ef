"""Learned NCA proposals: training data, GPU training, the shipped model.

The scoring network (per candidate point of an NCA block: 16 features ->
128 -> 128 -> 1, ReLU, BF16 weights, FP32 accumulation) is trained to
predict which points the NCA chooses as pivots. Training data comes from
plain NCA assemblies with the recorder on (features and pivot labels of every
block); training runs on the GPU through the library's own kernels
(h2w_mlp_grad, h2w_mlp_adam). The rank estimate of a block is
ceil(calib * sum of its rows' probabilities) + margin, calib fitted on the
training data.

    python -m h2weak_gb300.learned train --out model.npz
"""
import argparse
import ctypes
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MODEL = os.path.join(HERE, "data", "nca_mlp.npz")
F, H = 16, 128

# training problems: (dim, form, choice, tol, grid n | -npts uniform, nlevels)
# small relatives of the benchmark configurations (1D RBF, 2D IE/RBF, 3D RBF
# semi-nested, 3D IE) plus uniform random point sets
TRAIN_SET = [
    (1, 0, 1, 10, 8192, 7),
    (2, 0, 0, 10, 128, 4),
    (2, 0, 1, 10, 128, 4),
    (2, 0, 1, 8, -20000, 4),
    (2, 0, 0, 8, -12000, 4),
    (3, 1, 1, 8, 24, 3),
    (3, 0, 0, 8, 24, 3),
    (3, 0, 1, 10, -30000, 3),
]


def nparam():
    from h2weak_gb300 import lib
    return int(lib().h2w_mlp_nparam())


def init_params(seed=0):
    """He-normal weights, zero biases; layout W1, b1, W2, b2, w3, b3."""
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / F), (F, H))
    W2 = rng.normal(0, np.sqrt(2.0 / H), (H, H))
    w3 = rng.normal(0, np.sqrt(1.0 / H), H)
    p = np.concatenate([W1.ravel(), np.zeros(H), W2.ravel(), np.zeros(H), w3, [0.0]]).astype(np.float32)
    assert p.size == nparam()
    return p


def make_problem(hw, spec, device=0):
    from h2weak_gb300 import synth
    dim, form, choice, tol, n, nl = spec
    if n > 0:
        N = n ** dim
        op = hw.H2Operator(dim, form, choice, tol, nl, kernel_n=N, diag_n=2 * N if dim == 1 else N, device=device)
        op.gen_grid(n)
    else:
        op = hw.H2Operator(dim, form, choice, tol, nl, device=device)
        op.set_points(synth.uniform_points(synth.config_seed(6, -n), -n, dim))
    op.build_tree()
    return op


def collect(specs=TRAIN_SET, device=0):
    """Plain NCA assemblies with the recorder on: features and pivot labels."""
    import h2weak_gb300 as hw
    Xs, ys = [], []
    for spec in specs:
        op = make_problem(hw, spec, device)
        op.learn_record(True)
        op.assemble(hw.ASSEMBLE_NCA)
        X, y = op.learn_data()
        op.learn_record(False)
        Xs.append(X)
        ys.append(y)
        op.close()
    return np.concatenate(Xs), np.concatenate(ys)


def train(X, y, epochs=12, batch=65536, lr=2e-3, seed=0, params=None, log=None):
    """Adam on the GPU with the library's kernels; returns (params, losses)."""
    import torch
    import h2weak_gb300 as hw
    L = hw.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    n = len(y)
    pos = max(int(y.sum()), 1)
    pos_weight = float((n - pos) / pos)
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).to(dev)
    yd = torch.from_numpy(np.ascontiguousarray(y, dtype=np.uint8)).to(dev)
    p = torch.from_numpy(init_params(seed) if params is None else np.array(params, dtype=np.float32)).to(dev)
    g = torch.zeros_like(p)
    m = torch.zeros_like(p)
    v = torch.zeros_like(p)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    rng = np.random.default_rng(seed + 1)
    losses, step = [], 0
    torch.cuda.synchronize()
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).to(dev)
        tot = 0.0
        nb = 0
        for b0 in range(0, n, batch):
            sel = perm[b0:b0 + batch]
            xb = Xd[sel].contiguous()
            yb = yd[sel].contiguous()
            rc = L.h2w_mlp_grad(ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(xb.data_ptr()),
                                ctypes.c_void_p(yb.data_ptr()), len(sel), pos_weight, ctypes.c_void_p(g.data_ptr()),
                                ctypes.c_void_p(loss.data_ptr()), None)
            assert rc == 0
            step += 1
            rc = L.h2w_mlp_adam(ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(g.data_ptr()),
                                ctypes.c_void_p(m.data_ptr()), ctypes.c_void_p(v.data_ptr()), step, lr, None)
            assert rc == 0
            torch.cuda.synchronize()
            tot += float(loss.item())
            nb += 1
        losses.append(tot / nb)
        if log:
            log("epoch %d loss %.5f" % (ep, losses[-1]))
    return p.cpu().numpy(), losses


def logits(params, X):
    import torch
    import h2weak_gb300 as hw
    dev = torch.device("cuda", torch.cuda.current_device())
    p = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float32)).to(dev)
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).to(dev)
    z = torch.empty(len(X), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    assert hw.lib().h2w_mlp_forward(ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(Xd.data_ptr()), len(X),
                                    ctypes.c_void_p(z.data_ptr()), None) == 0
    torch.cuda.synchronize()
    return z.cpu().numpy()


def calibrate(params, X, y):
    """calib = (row pivots) / (sum of row probabilities) over the data."""
    z = logits(params, X)
    rows = X[:, 7] > 0.5
    prob = 1.0 / (1.0 + np.exp(-z[rows].astype(np.float64)))
    return float(y[rows].sum() / max(prob.sum(), 1e-30))


def save(path, params, calib, margin=2, info=None):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, params=np.asarray(params, dtype=np.float32), calib=np.float32(calib),
                        margin=np.int32(margin), info=json.dumps(info or {}))


def load(path=MODEL):
    d = np.load(path)
    return d["params"], float(d["calib"]), int(d["margin"])


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["train"])
    ap.add_argument("--out", default=MODEL)
    ap.add_argument("--epochs", type=int, default=12)
    a = ap.parse_args(argv)
    t0 = time.time()
    X, y = collect()
    t1 = time.time()
    params, losses = train(X, y, epochs=a.epochs, log=print)
    t2 = time.time()
    calib = calibrate(params, X, y)
    info = {"samples": int(len(y)), "positives": int(y.sum()), "losses": losses, "collect_s": t1 - t0,
            "train_s": t2 - t1, "calib": calib, "train_set": TRAIN_SET}
    save(a.out, params, calib, 2, info)
    print(json.dumps(info))


if __name__ == "__main__":
    main()
