"""CPU oracle of the learned-proposal network (test infrastructure only).

The network of h2weak_gb300's learned NCA proposals restated in float64
numpy: 16 -> 128 -> 128 -> 1 with ReLU, weights rounded to BF16 (round to
nearest even on the float32 bit pattern) as the GPU kernels use them, biases
as given; the mean weighted binary cross-entropy with logits and its
gradient by hand-written backpropagation. The GPU forward and gradient
kernels are checked against these functions.
"""
import numpy as np

F, H = 16, 128
SIZES = [("W1", F * H), ("b1", H), ("W2", H * H), ("b2", H), ("w3", H), ("b3", 1)]


def bf16(a):
    """float32 -> nearest BF16 (ties to even), returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    out, o = {}, 0
    dt = np.float64 if np.asarray(p).dtype == np.float64 else np.float32
    for name, n in SIZES:
        out[name] = np.asarray(p[o:o + n], dtype=dt)
        o += n
    assert o == len(p)
    return out


def forward(p, X, rounded=True):
    """Logits and the intermediate values; rounded=False keeps the weights
    unrounded (for finite-difference checks of the backpropagation)."""
    q = unpack(np.asarray(p, dtype=np.float64) if not rounded else p)
    rnd = bf16 if rounded else (lambda a: np.asarray(a, dtype=np.float64))
    W1, W2, w3 = rnd(q["W1"]).reshape(F, H), rnd(q["W2"]).reshape(H, H), rnd(q["w3"])
    b1, b2, b3 = q["b1"].astype(np.float64), q["b2"].astype(np.float64), float(q["b3"][0])
    X = np.asarray(X, dtype=np.float64)
    a1 = X @ W1 + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2 + b2
    h2 = np.maximum(a2, 0)
    z = h2 @ w3 + b3
    return z, (X, a1, h1, a2, h2, W1, W2, w3)


def loss_grad(p, X, y, pos_weight, rounded=True):
    z, (X, a1, h1, a2, h2, W1, W2, w3) = forward(p, X, rounded)
    y = np.asarray(y, dtype=np.float64)
    w = np.where(y > 0, pos_weight, 1.0)
    n = len(y)
    sp = np.where(z > 0, z + np.log1p(np.exp(-z)), np.log1p(np.exp(z)))
    loss = float(np.sum(w * (sp - y * z)) / n)
    dz = w * (1.0 / (1.0 + np.exp(-z)) - y) / n
    gw3 = h2.T @ dz
    gb3 = dz.sum()
    d2 = np.outer(dz, w3) * (a2 > 0)
    gW2 = h1.T @ d2
    gb2 = d2.sum(0)
    d1 = (d2 @ W2.T) * (a1 > 0)
    gW1 = X.T @ d1
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    return loss, g
