"""Double-precision restatement of the learned schedule's 16-64-64-2 network (forward, mean-squared-error
loss on the finite targets, gradients of every weight), in the weight layout of rsa_mpi_gb300/csrc/mlp.cu:
W1[64][16], b1[64], W2[64][64], b2[64], W3[2][64], b3[2].

TEST INFRASTRUCTURE ONLY: the checker of the GPU's forward and backward kernels.
"""
import numpy as np

NI, NH, NO = 16, 64, 2
SIZES = [("W1", (NH, NI)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NO, NH)), ("b3", (NO,))]
NW = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(w):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(w[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def bf16_to_f64(bits):
    return (np.asarray(bits, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def forward(w, x):
    p = unpack(w)
    x = np.asarray(x, dtype=np.float64)
    a1 = x @ p["W1"].T + p["b1"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ p["W2"].T + p["b2"]
    h2 = np.maximum(a2, 0)
    y = h2 @ p["W3"].T + p["b3"]
    return y, (x, a1, h1, a2, h2)


def loss_and_grad(w, x, t):
    y, (x, a1, h1, a2, h2) = forward(w, x)
    t = np.asarray(t, dtype=np.float64)
    valid = np.isfinite(t)
    nv = valid.sum()
    e = np.where(valid, y - np.where(valid, t, 0), 0.0)
    loss = (e * e).sum() / nv
    dy = 2 * e / nv
    p = unpack(w)
    gW3 = dy.T @ h2
    gb3 = dy.sum(0)
    dh2 = (dy @ p["W3"]) * (a2 > 0)
    gW2 = dh2.T @ h1
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ p["W2"]) * (a1 > 0)
    gW1 = dh1.T @ x
    gb1 = dh1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
