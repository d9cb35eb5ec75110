"""CPU oracle of the opening-policy network (TEST INFRASTRUCTURE ONLY): forward pass, mean-squared
error and its gradient, and one Adam step, in float64 numpy, for checking the GPU training
kernels. Parameter layout as in include/nbody.h: W1[8][32], b1[32], W2[32][32], b2[32], w3[32], b3.
"""

import numpy as np

SHAPES = [("W1", (8, 32)), ("b1", (32,)), ("W2", (32, 32)), ("b2", (32,)), ("w3", (32,)),
          ("b3", (1,))]
COUNT = 1377


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, k = {}, 0
    for name, shape in SHAPES:
        size = int(np.prod(shape))
        out[name] = p[k:k + size].reshape(shape)
        k += size
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def forward(p, X):
    w = unpack(p)
    a1 = X @ w["W1"] + w["b1"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ w["W2"] + w["b2"]
    h2 = np.maximum(a2, 0)
    out = h2 @ w["w3"] + w["b3"][0]
    return out, (a1, h1, a2, h2)


def loss_grad(p, X, Y):
    """Mean squared error over the rows and its gradient with respect to the parameters."""
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    w = unpack(p)
    out, (a1, h1, a2, h2) = forward(p, X)
    n = len(Y)
    e = out - Y
    loss = np.mean(e * e)
    dout = 2 * e / n
    g = {"w3": h2.T @ dout, "b3": np.array([dout.sum()])}
    d2 = np.outer(dout, w["w3"]) * (a2 > 0)
    g["W2"] = h1.T @ d2
    g["b2"] = d2.sum(axis=0)
    d1 = (d2 @ w["W2"].T) * (a1 > 0)
    g["W1"] = X.T @ d1
    g["b1"] = d1.sum(axis=0)
    return loss, pack(g)


def adam_step(p, m, v, g, lr, b1, b2, eps, t):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
