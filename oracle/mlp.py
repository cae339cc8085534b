"""CPU oracle of the cost-model MLP (TEST INFRASTRUCTURE).

numpy restatement of the engine's hand-written CUDA kernels for the learned
cost model (ttv_gb300/csrc/ttv_mlp.cu): the same flat parameter layout
  W1[IN][H] b1[H] W2[H][H] b2[H] W3[H][H] b3[H] W4[H] b4
with three ReLU hidden layers of 64 units, the loss
  L = (1/n) sum_s 0.5 (f(x_s) - y_s)^2
its analytic gradient (float64), and one Adam step.  The GPU gradients are
checked against this, and this against central finite differences.
"""
from __future__ import annotations

import numpy as np

IN, H = 17, 64
SIZES = [("W1", (IN, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)),
         ("b3", (H,)), ("W4", (H,)), ("b4", (1,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(params):
    out, o = {}, 0
    p = np.asarray(params, dtype=np.float64)
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def forward(params, x):
    w = unpack(params)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ w["W1"] + w["b1"]
    a1 = np.maximum(z1, 0)
    z2 = a1 @ w["W2"] + w["b2"]
    a2 = np.maximum(z2, 0)
    z3 = a2 @ w["W3"] + w["b3"]
    a3 = np.maximum(z3, 0)
    out = a3 @ w["W4"] + w["b4"][0]
    return out, (x, z1, a1, z2, a2, z3, a3)


def loss(params, x, y):
    out, _ = forward(params, x)
    return float(np.sum(0.5 * (out - y) ** 2) / len(y))


def loss_grad(params, x, y):
    w = unpack(params)
    out, (x, z1, a1, z2, a2, z3, a3) = forward(params, x)
    n = len(y)
    dout = (out - np.asarray(y, dtype=np.float64)) / n
    g = {"W4": a3.T @ dout, "b4": np.array([dout.sum()])}
    d3 = np.outer(dout, w["W4"]) * (z3 > 0)
    g["W3"] = a2.T @ d3
    g["b3"] = d3.sum(0)
    d2 = (d3 @ w["W3"].T) * (z2 > 0)
    g["W2"] = a1.T @ d2
    g["b2"] = d2.sum(0)
    d1 = (d2 @ w["W2"].T) * (z1 > 0)
    g["W1"] = x.T @ d1
    g["b1"] = d1.sum(0)
    L = float(np.sum(0.5 * (out - y) ** 2) / n)
    return L, pack(g)


def adam(params, grad, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mhat = m / (1 - b1 ** step)
    vhat = v / (1 - b2 ** step)
    return params - lr * mhat / (np.sqrt(vhat) + eps), m, v
