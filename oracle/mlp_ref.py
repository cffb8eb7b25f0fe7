"""FP64 numpy restatement of the learned-alpha network and its gradient
(test infrastructure: the checker of the GPU training kernels).

Network: x (27) -> GELU(x W1 + b1) (64) -> GELU(h1 W2 + b2) (64) -> h2 . w3 + b3,
GELU in its tanh form; loss = mean over the batch of (out - target)^2.
Parameter layout (6017): W1[27][64], b1[64], W2[64][64], b2[64], w3[64], b3.
"""
from __future__ import annotations

import numpy as np

NI, NH = 27, 64
SIZES = [("W1", (NI, NH)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("w3", (NH,)), ("b3", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)
K0, K1 = 0.7978845608028654, 0.044715


def unpack(w):
    out, o = {}, 0
    for name, shp in SIZES:
        n = int(np.prod(shp))
        out[name] = np.asarray(w[o:o + n], np.float64).reshape(shp)
        o += n
    return out


def pack(parts):
    return np.concatenate([np.asarray(parts[n], np.float64).ravel() for n, _ in SIZES])


def gelu(z):
    t = np.tanh(K0 * (z + K1 * z ** 3))
    g = 0.5 * z * (1 + t)
    dg = 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * K0 * (1 + 3 * K1 * z * z)
    return g, dg


def init(seed=0):
    rng = np.random.default_rng(seed)
    p = {"W1": rng.normal(0, 1 / np.sqrt(NI), (NI, NH)), "b1": np.zeros(NH),
         "W2": rng.normal(0, 1 / np.sqrt(NH), (NH, NH)), "b2": np.zeros(NH),
         "w3": rng.normal(0, 1 / np.sqrt(NH), NH), "b3": np.zeros(1)}
    return pack(p)


def forward(w, x):
    p = unpack(w)
    z1 = x @ p["W1"] + p["b1"]
    h1, d1 = gelu(z1)
    z2 = h1 @ p["W2"] + p["b2"]
    h2, d2 = gelu(z2)
    out = h2 @ p["w3"] + p["b3"][0]
    return out, (x, h1, d1, h2, d2)


def loss_and_grad(w, rec):
    rec = np.asarray(rec, np.float64)
    x, t = rec[:, :NI], rec[:, NI + 1]
    out, (x, h1, d1, h2, d2) = forward(w, x)
    n = x.shape[0]
    err = out - t
    loss = np.mean(err ** 2)
    dout = 2 * err / n
    p = unpack(w)
    dz2 = dout[:, None] * p["w3"][None, :] * d2
    dz1 = (dz2 @ p["W2"].T) * d1
    g = {"W1": x.T @ dz1, "b1": dz1.sum(0), "W2": h1.T @ dz2, "b2": dz2.sum(0), "w3": h2.T @ dout,
         "b3": np.array([dout.sum()])}
    return loss, pack(g)
