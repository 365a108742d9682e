"""FP64 NumPy reference of the cooling-function surrogate network.

TEST INFRASTRUCTURE ONLY: the CPU oracle that the GPU training kernels'
losses and gradients are checked against.  Parameter layout as in
include/galnode_surrogate.h: W1[64][3], b1, W2[64][64], b2, W3[64][64], b3,
W4[64], b4; SiLU activations; loss = mean squared error.
"""

import numpy as np

SIZES = [("W1", (64, 3)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (64, 64)), ("b3", (64,)),
         ("W4", (64,)), ("b4", (1,))]


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x):
    w = unpack(p)
    z1 = x @ w["W1"].T + w["b1"]
    a1 = silu(z1)
    z2 = a1 @ w["W2"].T + w["b2"]
    a2 = silu(z2)
    z3 = a2 @ w["W3"].T + w["b3"]
    a3 = silu(z3)
    out = a3 @ w["W4"] + w["b4"][0]
    return out, (z1, a1, z2, a2, z3, a3)


def loss_and_gradient(p, x, y):
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(y)
    w = unpack(p)
    out, (z1, a1, z2, a2, z3, a3) = forward(p, x)
    r = out - y
    loss = np.mean(r * r)
    dout = 2.0 * r / n
    g = {"W4": a3.T @ dout, "b4": np.array([dout.sum()])}
    dz3 = np.outer(dout, w["W4"]) * silu_grad(z3)
    g["W3"] = dz3.T @ a2
    g["b3"] = dz3.sum(axis=0)
    dz2 = (dz3 @ w["W3"]) * silu_grad(z2)
    g["W2"] = dz2.T @ a1
    g["b2"] = dz2.sum(axis=0)
    dz1 = (dz2 @ w["W2"]) * silu_grad(z1)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(axis=0)
    return loss, pack(g)
