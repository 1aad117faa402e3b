"""FP64 CPU restatement of the cost model's network (test infrastructure only).

The engine's MLP (quant-iron_gb300/csrc/qi_mlp.cu) has no reference
counterpart; this numpy FP64 forward/backward is the oracle its GPU
gradients are checked against.  Parameter layout (flat vector): for each
layer l = 0..3, W_l [out][in] row-major then b_l [out]; sizes 20->64->64->64->1,
ReLU on the hidden layers, loss = mean((pred - y)^2).
"""
import numpy as np

SIZES = [(20, 64), (64, 64), (64, 64), (64, 1)]


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, off = [], 0
    for i, o in SIZES:
        W = p[off:off + i * o].reshape(o, i)
        off += i * o
        b = p[off:off + o]
        off += o
        out.append((W, b))
    assert off == p.size
    return out


def loss_and_gradient(p, X, y):
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    layers = unpack(p)
    acts, zs = [X], []
    a = X
    for li, (W, b) in enumerate(layers):
        z = a @ W.T + b
        zs.append(z)
        a = np.maximum(z, 0.0) if li < 3 else z
        acts.append(a)
    pred = a[:, 0]
    n = y.size
    loss = np.mean((pred - y) ** 2)
    d = (2.0 * (pred - y) / n)[:, None]
    grads = []
    for li in range(3, -1, -1):
        W, b = layers[li]
        if li < 3:
            d = d * (zs[li] > 0)
        gW = d.T @ acts[li]
        gb = d.sum(axis=0)
        grads.append((gW, gb))
        d = d @ W
    flat = []
    for gW, gb in reversed(grads):
        flat.append(gW.reshape(-1))
        flat.append(gb)
    return loss, np.concatenate(flat)
